// Drop-in replacements for the reference's two native kernels
// (gbgpu/cutils/gbgpu_utils.cu): batched <d|h>, <h|h> over point-major
// templates, and the scatter-add of templates into global buffers.
// get_ll: one warp per two binaries (lanes interleaved by binary); fill: one
// warp per binary, lanes along the window.
#include <cuda.h>            // CUtensorMap (the type; the encoder comes through the runtime)
#include <cudaTypedefs.h>

#include <mutex>

#include "gbx_common.cuh"
#include "gbx_internal.h"

namespace gbx {

// conj(d) h w and |h|^2 w of one bin of one channel, accumulated into the
// float pairs dr, di, hh
__device__ __forceinline__ void ll_bin(double2 d, double2 hv, double S, int eD, int eS, dfl &dr,
                                       dfl &di, dfl &hh)
{
    const dfl dR = d2ff_scaled(d.x, eD), dI = d2ff_scaled(d.y, eD);
    const dfl hR = d2ff_scaled(hv.x, eD), hI = d2ff_scaled(hv.y, eD);
    const dfl w = df_recip(d2ff_scaled(S, eS));
    const dfl re = df_sum(df_prod(dR, hR), df_prod(dI, hI));
    const dfl im = df_sum(df_prod(dR, hI), df_neg(df_prod(dI, hR)));
    const dfl sq = df_sum(df_prod(hR, hR), df_prod(hI, hI));
    dr = df_add(dr, df_prod(re, w));         // accumulators stay normalised
    di = df_add(di, df_prod(im, w));
    hh = df_add(hh, df_prod(sq, w));
}

// sum over the 16 lanes of the same parity (the lanes of one binary)
__device__ __forceinline__ dfl pair_sum_df(dfl v)
{
#pragma unroll
    for (int o = 16; o > 1; o >>= 1) {
        const dfl y = {__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
        v = df_add(v, y);
    }
    return v;
}

// <d|h>, <h|h> per binary (gbgpu_utils.cu:124-210).  A warp takes two
// binaries: lane 2q + t walks points q, q + 16, ... of binary b + t, so a
// warp's template loads cover whole 32-byte sectors in the point-major layout
// (the two binaries' elements are adjacent) and its data and PSD loads are
// two contiguous runs.  The FP64 inputs are split into float pairs with
// per-binary power-of-two scalings (S 2^eS and d 2^eD of order one, from the
// PSD at the window centre) and multiplied and summed as float pairs on the
// FP32 pipe (about 46 significant bits: each sum is within ~1e-13 of
// sum |terms| of the FP64 result); one FP64 conversion per output.  A
// negative row, or one at or above num_data / num_psd when those are
// positive, is flagged (GBX_FLAG_INDEX), never read, and gives zero outputs.
__global__ void __launch_bounds__(256) get_ll_kernel(
    double2 *__restrict__ d_h, double2 *__restrict__ h_h, const double2 *__restrict__ A_t,
    const double2 *__restrict__ E_t, const double2 *__restrict__ A_d,
    const double2 *__restrict__ E_d, const double *__restrict__ A_p,
    const double *__restrict__ E_p, double df, const int *__restrict__ start_ind, int M,
    int num_bin, const int *__restrict__ data_index, const int *__restrict__ noise_index,
    int L, long long tsi, long long tsb, int num_data, int num_psd, int *status)
{
    const int lane = threadIdx.x & 31, t = lane & 1, q = lane >> 1;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int b0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2; b0 < num_bin; b0 += 2 * warps) {
        const int b = b0 + t;
        const bool has = b < num_bin;                 // odd num_bin: the last warp's lane t = 1 idles
        const int s = has ? start_ind[b] : 0;
        const int drow = has && data_index ? data_index[b] : 0;
        const int nrow = has && noise_index ? noise_index[b] : 0;
        const bool bad = drow < 0 || nrow < 0 || (num_data > 0 && drow >= num_data) ||
                         (num_psd > 0 && nrow >= num_psd);
        if (bad && q == 0) flag(status, GBX_FLAG_INDEX);
        const bool use = has && !bad;
        const size_t doff = (size_t)(use ? drow : 0) * L;
        const size_t noff = (size_t)(use ? nrow : 0) * L;
        int jm = s + M / 2;
        jm = jm < 0 ? 0 : (jm >= L ? L - 1 : jm);
        // exponent of the PSD at the window centre, on the integer pipe
        // (0 for zero, negative, subnormal or non-finite values)
        const int hS = L > 0 && use ? __double2hiint(__ldg(A_p + noff + jm)) : 0;
        const int exS = (hS >> 20) & 0x7ff;
        const int lgS = (hS > 0 && exS > 0 && exS < 0x7ff) ? exS - 1023 : 0;
        const int eS = -lgS, eD = -(lgS >> 1) - 14;
        dfl dr = {0.f, 0.f}, di = {0.f, 0.f}, hh = {0.f, 0.f};
        bool out = false;
        const int Mh = use ? M : 0;
#pragma unroll 2
        for (int i = q; i < Mh; i += 16) {
            const int j = s + i;
            if (j < 0 || j >= L) {
                out = true;
                continue;
            }
            const double2 hA = __ldg(A_t + i * tsi + b * tsb);
            const double2 hE = __ldg(E_t + i * tsi + b * tsb);
            const double2 dA = __ldg(A_d + doff + j), dE = __ldg(E_d + doff + j);
            const double SA = __ldg(A_p + noff + j), SE = __ldg(E_p + noff + j);
            ll_bin(dA, hA, SA, eD, eS, dr, di, hh);
            ll_bin(dE, hE, SE, eD, eS, dr, di, hh);
        }
        dr = pair_sum_df(dr);
        di = pair_sum_df(di);
        hh = pair_sum_df(hh);
        if (__any_sync(0xffffffffu, out) && lane == 0) flag(status, GBX_FLAG_WINDOW);
        if (q == 0 && has) {
            // undo the scalings: terms carry 2^(2 eD - eS)
            const double s4 = 4. * df * __hiloint2double((eS - 2 * eD + 1023) << 20, 0);
            d_h[b] = make_double2(s4 * ((double)dr.h + (double)dr.l),
                                  s4 * ((double)di.h + (double)di.l));
            h_h[b] = make_double2(s4 * ((double)hh.h + (double)hh.l), 0.0);
        }
    }
}

// ---------------------------------------------------------------------------
// get_ll with every input staged in shared memory by asynchronous copies
// completing on an mbarrier: the templates by TMA tensor copies (a box of the
// pair's two binaries x kBulkC points, from a 2-D tensor map over the template
// array, point-major or binary-major), the data and PSD windows by bulk copies
// (cp.async.bulk).  Same warp layout and arithmetic as get_ll_kernel; each
// warp walks its binary pairs in chunks of kBulkC points and keeps two chunk
// buffers in flight, so one lane issues every load ahead of use and no lane
// waits on a global load.  A PSD chunk is copied from the even element at or
// below its first bin (16-byte alignment of the copy), and an odd last element
// is read directly.  Waits are bounded: on a timeout the warp sets
// GBX_FLAG_TIMEOUT, waits (bounded) for its copies in flight and stops.
constexpr int kBulkC = 64;                 // points per binary per chunk
constexpr int kBulkWarps = 4;              // warps per CTA
constexpr int kSpinLimit = 1 << 16;        // polls of a barrier before giving up

struct __align__(128) BulkBuf {
    double2 h[2][2 * kBulkC];              // [A, E]: template box, [point][binary] or [binary][point]
    double2 d[2][2][kBulkC];               // [binary][A, E][point]: data
    double p[2][2][kBulkC + 2];            // [binary][A, E][element]: PSD from an even element
};

__device__ __forceinline__ unsigned smem_addr(const void *ptr)
{
    return (unsigned)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// bounded wait for the phase of the given parity, agreed by the whole warp
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity)
{
    bool ok = false;
    for (int i = 0; i < kSpinLimit && !ok; i++) ok = mbar_try(bar, parity);
    return __all_sync(0xffffffffu, ok);
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes,
                                          unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tensor_load(void *dst, const CUtensorMap *map, int x, int y,
                                            unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(smem_addr(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y),
                   "r"(smem_addr(bar)) : "memory");
}

// the bins of chunk c of a binary with window start s that lie in [0, L):
// [lo, hi), and the PSD elements (absolute indices) copied for them: [pa, pe)
struct BulkRange {
    int jc, lo, hi;
    long long base, pa, pe;
};

__device__ __forceinline__ BulkRange bulk_range(int s, int c, int M, int L, long long noff)
{
    BulkRange r;
    r.jc = s + c * kBulkC;
    r.lo = max(r.jc, 0);
    r.hi = min(min(r.jc + kBulkC, s + M), L);
    r.base = (noff + r.jc) & ~1LL;
    r.pa = (noff + r.lo) & ~1LL;
    r.pe = r.hi > r.lo ? ((noff + r.hi) & ~1LL) : r.pa;
    return r;
}

// layout 0: point-major templates (element i * num_bin + b), layout 1:
// binary-major (element b * M + i); the tensor maps tmA / tmE match it
__global__ void __launch_bounds__(kBulkWarps * 32) get_ll_bulk_kernel(
    double2 *__restrict__ d_h, double2 *__restrict__ h_h, const __grid_constant__ CUtensorMap tmA,
    const __grid_constant__ CUtensorMap tmE, int layout, const double2 *__restrict__ A_d,
    const double2 *__restrict__ E_d, const double *__restrict__ A_p,
    const double *__restrict__ E_p, double df, const int *__restrict__ start_ind, int M,
    int num_bin, const int *__restrict__ data_index, const int *__restrict__ noise_index,
    int L, int num_data, int num_psd, int *status)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, t = lane & 1, q = lane >> 1;
    BulkBuf *buf = reinterpret_cast<BulkBuf *>(smem) + 2 * warp;
    unsigned long long *bar =
        reinterpret_cast<unsigned long long *>(smem + sizeof(BulkBuf) * 2 * kBulkWarps) + 2 * warp;
    if (lane == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    const int nw = gridDim.x * kBulkWarps;
    const int gw = blockIdx.x * kBulkWarps + warp;
    const int npair = (num_bin + 1) / 2;
    const int nchunk = (M + kBulkC - 1) / kBulkC;
    const int mypairs = gw < npair ? (npair - gw + nw - 1) / nw : 0;
    const int K = mypairs * nchunk;
    constexpr unsigned kBoxBytes = 2 * kBulkC * sizeof(double2);   // one template box

    // rows of binary b (false when out of range: nothing is read for it)
    auto rows = [&](int b, size_t &doff, size_t &noff) {
        const int dr = data_index ? data_index[b] : 0;
        const int nr = noise_index ? noise_index[b] : 0;
        const bool ok = dr >= 0 && nr >= 0 && (num_data <= 0 || dr < num_data) &&
                        (num_psd <= 0 || nr < num_psd);
        doff = (size_t)(ok ? dr : 0) * L;
        noff = (size_t)(ok ? nr : 0) * L;
        return ok;
    };
    // copy item k (pair gw + (k / nchunk) nw, chunk k % nchunk) into buffer
    // slot, issued by lanes 0-3 together: lane u < 2 the data and PSD windows
    // of binary u, lane 2 / 3 the template box of A / E, lane 0 the
    // expected byte count (the transfers may complete before it is posted:
    // the phase needs that arrival too)
    auto issue = [&](int k, int slot) {
        const int pr = gw + (k / nchunk) * nw, c = k % nchunk;
        BulkBuf &B = buf[slot];
        unsigned bytes = 0;
        if (lane < 2) {
            const int u = lane, b = 2 * pr + u;
            size_t doff = 0, noff = 0;
            if (b < num_bin && rows(b, doff, noff)) {
                const BulkRange r = bulk_range(start_ind[b], c, M, L, (long long)noff);
                const int n = max(r.hi - r.lo, 0);
                const long long pn = r.pe - r.pa;
                bytes = 2u * (16u * n + 8u * (unsigned)pn);
                if (n > 0) {
                    bulk_load(&B.d[u][0][r.lo - r.jc], A_d + doff + r.lo, 16u * n, &bar[slot]);
                    bulk_load(&B.d[u][1][r.lo - r.jc], E_d + doff + r.lo, 16u * n, &bar[slot]);
                }
                if (pn > 0) {
                    bulk_load(&B.p[u][0][r.pa - r.base], A_p + r.pa, 8u * (unsigned)pn, &bar[slot]);
                    bulk_load(&B.p[u][1][r.pa - r.base], E_p + r.pa, 8u * (unsigned)pn, &bar[slot]);
                }
            }
        } else if (lane < 4) {
            // template boxes: inner coordinate in doubles (a multiple of 2, i.e.
            // 16 bytes); points or binaries past the array are filled with zeros
            const int x = layout == 0 ? 4 * pr : 2 * c * kBulkC;
            const int y = layout == 0 ? c * kBulkC : 2 * pr;
            tensor_load(&B.h[lane - 2][0], lane == 2 ? &tmA : &tmE, x, y, &bar[slot]);
        }
        bytes += __shfl_xor_sync(0x0000000fu, bytes, 1);
        if (lane == 0) mbar_expect(&bar[slot], bytes + 2 * kBoxBytes);
    };

    if (lane < 4) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (K > 0) issue(0, 0);
        if (K > 1) issue(1, 1);
    }
    dfl dr = {0.f, 0.f}, di = {0.f, 0.f}, hh = {0.f, 0.f};
    bool out = false;
    int s = 0, eS = 0, eD = 0, b = 0;
    size_t doff = 0, noff = 0;
    bool use = false;
    for (int k = 0; k < K; k++) {
        const int slot = k & 1;
        const int pr = gw + (k / nchunk) * nw, c = k % nchunk;
        if (c == 0) {
            b = 2 * pr + t;
            use = b < num_bin;
            if (use) {
                const bool ok = rows(b, doff, noff);
                if (!ok && q == 0) flag(status, GBX_FLAG_INDEX);
                use = ok;
                s = start_ind[b];
                int jm = s + M / 2;
                jm = jm < 0 ? 0 : (jm >= L ? L - 1 : jm);
                const int hS = use ? __double2hiint(__ldg(A_p + noff + jm)) : 0;
                const int exS = (hS >> 20) & 0x7ff;
                const int lgS = (hS > 0 && exS > 0 && exS < 0x7ff) ? exS - 1023 : 0;
                eS = -lgS;
                eD = -(lgS >> 1) - 14;
            }
        }
        if (!mbar_wait(&bar[slot], (unsigned)(k >> 1) & 1u)) {
            if (lane == 0) flag(status, GBX_FLAG_TIMEOUT);
            // the copies still in flight target this warp's buffers: wait for
            // them (bounded) before the warp stops
            mbar_wait(&bar[slot], (unsigned)(k >> 1) & 1u);
            if (K > k + 1) mbar_wait(&bar[slot ^ 1], (unsigned)((k + 1) >> 1) & 1u);
            return;
        }
        const BulkBuf &B = buf[slot];
        if (use) {
            const BulkRange r = bulk_range(s, c, M, L, (long long)noff);
#pragma unroll
            for (int m = 0; m < kBulkC / 16; m++) {
                const int i = q + 16 * m, ip = c * kBulkC + i;
                if (ip >= M) break;
                const int j = s + ip;
                if (j < 0 || j >= L) {
                    out = true;
                    continue;
                }
                const long long e = (long long)noff + j;
                const bool in = e < r.pe;
                const double SA = in ? B.p[t][0][e - r.base] : __ldg(A_p + e);
                const double SE = in ? B.p[t][1][e - r.base] : __ldg(E_p + e);
                const int hi = layout == 0 ? 2 * i + t : t * kBulkC + i;
                ll_bin(B.d[t][0][i], B.h[0][hi], SA, eD, eS, dr, di, hh);
                ll_bin(B.d[t][1][i], B.h[1][hi], SE, eD, eS, dr, di, hh);
            }
        }
        __syncwarp();
        if (lane < 4 && k + 2 < K) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k + 2, slot);
        }
        if (c == nchunk - 1) {
            dr = pair_sum_df(dr);
            di = pair_sum_df(di);
            hh = pair_sum_df(hh);
            if (__any_sync(0xffffffffu, out) && lane == 0) flag(status, GBX_FLAG_WINDOW);
            if (q == 0 && b < num_bin) {
                const double s4 = 4. * df * __hiloint2double((eS - 2 * eD + 1023) << 20, 0);
                d_h[b] = use ? make_double2(s4 * ((double)dr.h + (double)dr.l),
                                            s4 * ((double)di.h + (double)di.l))
                             : make_double2(0.0, 0.0);
                h_h[b] = use ? make_double2(s4 * ((double)hh.h + (double)hh.l), 0.0)
                             : make_double2(0.0, 0.0);
            }
            dr = di = hh = dfl{0.f, 0.f};
            out = false;
        }
    }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// to the driver library; NULL when the driver does not provide it)
static PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool tried = false;
    static std::mutex lock;
    std::lock_guard<std::mutex> g(lock);
    if (!tried) {
        tried = true;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        void *ptr = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    }
    return fn;
}

// 2-D tensor map over a complex128 template array seen as doubles: layout 0
// (point-major, num_bin x M) boxes 2 binaries x kBulkC points, layout 1
// (binary-major) boxes kBulkC points x 2 binaries
static bool make_template_map(CUtensorMap *map, const void *base, int layout, int num_bin, int M)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
    if (!enc || ((uintptr_t)base & 15) != 0) return false;
    cuuint64_t dims[2], strides[1];
    cuuint32_t box[2], es[2] = {1, 1};
    if (layout == 0) {
        dims[0] = 2ull * num_bin;
        dims[1] = (cuuint64_t)M;
        strides[0] = 16ull * num_bin;
        box[0] = 4;
        box[1] = kBulkC;
    } else {
        dims[0] = 2ull * M;
        dims[1] = (cuuint64_t)num_bin;
        strides[0] = 16ull * M;
        box[0] = 2 * kBulkC;
        box[1] = 2;
    }
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void *>(base), dims, strides, box,
               es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

__global__ void __launch_bounds__(256) fill_global_kernel(
    double2 *__restrict__ A_g, double2 *__restrict__ E_g, const double2 *__restrict__ A_t,
    const double2 *__restrict__ E_t, const int *__restrict__ start_ind, int M, int num_bin,
    const int *__restrict__ group_index, int L, long long gstride, long long tsi, long long tsb,
    int num_groups, int *status)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < num_bin; b += warps) {
        const int s = start_ind[b];
        const int g = group_index[b];
        if (num_groups > 0 && (g < 0 || g >= num_groups)) {
            if (lane == 0) flag(status, GBX_FLAG_INDEX);
            continue;
        }
        const size_t goff = (size_t)g * gstride;
        for (int i = lane; i < M; i += 32) {
            const int j = s + i;
            if (j < 0 || j >= L) continue;    // gbgpu_utils.cu:88-91
            const double2 a = __ldg(A_t + i * tsi + b * tsb);
            const double2 e = __ldg(E_t + i * tsi + b * tsb);
            atomicAdd(&A_g[goff + j].x, a.x);
            atomicAdd(&A_g[goff + j].y, a.y);
            atomicAdd(&E_g[goff + j].x, e.x);
            atomicAdd(&E_g[goff + j].y, e.y);
        }
    }
}

// Deterministic fill: one CTA per (chunk of kDetChunk output bins, group).
// Binaries of a group are visited in the order given by `order` (sorted by
// start index), so every output bin is the same sum in the same order on
// every run; every bin of channels A/E is written (zero where no window
// reaches), which is the reference's overwrite semantics (gbgpu.py:796-837).
constexpr int kDetChunk = 1024;
constexpr int kDetThreads = 256;

__global__ void __launch_bounds__(kDetThreads) fill_det_kernel(
    double2 *__restrict__ A_g, double2 *__restrict__ E_g, const double2 *__restrict__ A_t,
    const double2 *__restrict__ E_t, const int *__restrict__ start_ind, int M,
    const int *__restrict__ order, const int *__restrict__ group_first, int L, long long gstride,
    long long tsi, long long tsb)
{
    __shared__ int s_lo, s_hi;
    const int g = blockIdx.y;
    const int c0 = blockIdx.x * kDetChunk;
    if (threadIdx.x == 0) {
        // binaries whose window [s, s + M) meets [c0, c0 + kDetChunk): s in [c0 - M + 1, c0 + kDetChunk)
        const int b0 = group_first[g], b1 = group_first[g + 1];
        int lo = b0, hi = b1;
        const long long want_lo = (long long)c0 - M + 1;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if ((long long)start_ind[order[mid]] < want_lo) lo = mid + 1; else hi = mid;
        }
        s_lo = lo;
        int lo2 = lo, hi2 = b1;
        const long long want_hi = (long long)c0 + kDetChunk;
        while (lo2 < hi2) {
            const int mid = (lo2 + hi2) >> 1;
            if ((long long)start_ind[order[mid]] < want_hi) lo2 = mid + 1; else hi2 = mid;
        }
        s_hi = lo2;
    }
    __syncthreads();
    constexpr int PER = kDetChunk / kDetThreads;
    double2 a[PER], e[PER];
#pragma unroll
    for (int k = 0; k < PER; k++) {
        a[k] = make_double2(0.0, 0.0);
        e[k] = make_double2(0.0, 0.0);
    }
    for (int q = s_lo; q < s_hi; q++) {
        const int b = order[q];
        const int s = start_ind[b];
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const int j = c0 + threadIdx.x + k * kDetThreads;
            const int i = j - s;
            if (i >= 0 && i < M) {
                const double2 x = __ldg(A_t + i * tsi + b * tsb);
                const double2 y = __ldg(E_t + i * tsi + b * tsb);
                a[k].x += x.x; a[k].y += x.y;
                e[k].x += y.x; e[k].y += y.y;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < PER; k++) {
        const int j = c0 + threadIdx.x + k * kDetThreads;
        if (j < L) {
            A_g[(size_t)g * gstride + j] = a[k];
            E_g[(size_t)g * gstride + j] = e[k];
        }
    }
}

static int grid_for(int num_bin)
{
    int blocks = (num_bin + 7) / 8;
    int cap = num_sms() * 8;
    return blocks < cap ? (blocks > 0 ? blocks : 1) : cap;
}

}  // namespace gbx

using namespace gbx;

extern "C" int gbx_get_ll_ex(void *d_h, void *h_h, const void *A_template,
                             const void *E_template, const void *A_data, const void *E_data,
                             const double *A_psd, const double *E_psd, double df,
                             const int *start_ind, int M, int num_bin, const int *data_index,
                             const int *noise_index, int data_length, long long t_stride_i,
                             long long t_stride_b, int num_data, int num_psd, int *status,
                             void *stream)
{
    if (num_bin < 0 || M < 0 || data_length < 0) return set_error(GBX_ERR_ARG, "negative size");
    if (num_bin == 0) return GBX_OK;
    if (!d_h || !h_h || !A_template || !E_template || !A_data || !E_data || !A_psd || !E_psd ||
        !start_ind)
        return set_error(GBX_ERR_ARG, "NULL pointer");
    int rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    // staged kernel: 16-byte aligned data and PSD, point-major or binary-major
    // templates with tensor maps; anything else takes the direct-load kernel
    const bool aligned = ((uintptr_t)A_data | (uintptr_t)E_data | (uintptr_t)A_psd |
                          (uintptr_t)E_psd) % 16 == 0;
    const int layout = (t_stride_i == num_bin && t_stride_b == 1) ? 0
                     : (t_stride_i == 1 && t_stride_b == M) ? 1 : -1;
    CUtensorMap tmA, tmE;
    if (aligned && layout >= 0 && M > 0 && data_length > 0 &&
        make_template_map(&tmA, A_template, layout, num_bin, M) &&
        make_template_map(&tmE, E_template, layout, num_bin, M)) {
        auto kern = get_ll_bulk_kernel;
        const size_t sm = sizeof(BulkBuf) * 2 * kBulkWarps + 16 * kBulkWarps;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(get_ll_bulk)");
        int per_sm = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBulkWarps * 32, sm);
        if (e != cudaSuccess) return cuda_error(e, "occupancy(get_ll_bulk)");
        const int npair = (num_bin + 1) / 2;
        int grid = (per_sm > 0 ? per_sm : 1) * num_sms();
        const int need = (npair + kBulkWarps - 1) / kBulkWarps;
        if (grid > need) grid = need;
        kern<<<grid, kBulkWarps * 32, sm, (cudaStream_t)stream>>>(
            (double2 *)d_h, (double2 *)h_h, tmA, tmE, layout, (const double2 *)A_data,
            (const double2 *)E_data, A_psd, E_psd, df, start_ind, M, num_bin, data_index,
            noise_index, data_length, num_data, num_psd, status);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_error(e, "get_ll_bulk launch");
        return GBX_OK;
    }
    get_ll_kernel<<<grid_for((num_bin + 1) / 2), 256, 0, (cudaStream_t)stream>>>(
        (double2 *)d_h, (double2 *)h_h, (const double2 *)A_template, (const double2 *)E_template,
        (const double2 *)A_data, (const double2 *)E_data, A_psd, E_psd, df, start_ind, M, num_bin,
        data_index, noise_index, data_length, t_stride_i, t_stride_b, num_data, num_psd, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "get_ll launch");
    return GBX_OK;
}

extern "C" int gbx_get_ll(void *d_h, void *h_h, const void *A_template, const void *E_template,
                          const void *A_data, const void *E_data, const double *A_psd,
                          const double *E_psd, double df, const int *start_ind, int M,
                          int num_bin, const int *data_index, const int *noise_index,
                          int data_length, int *status, void *stream)
{
    return gbx_get_ll_ex(d_h, h_h, A_template, E_template, A_data, E_data, A_psd, E_psd, df,
                         start_ind, M, num_bin, data_index, noise_index, data_length,
                         (long long)num_bin, 1LL, 0, 0, status, stream);
}

extern "C" int gbx_fill_global_ex(void *A_glob, void *E_glob, const void *A_template,
                                  const void *E_template, const int *start_ind, int M,
                                  int num_bin, const int *group_index, int data_length,
                                  int num_groups, long long group_stride, long long t_stride_i,
                                  long long t_stride_b, int *status, void *stream)
{
    if (num_bin < 0 || M < 0 || data_length < 0) return set_error(GBX_ERR_ARG, "negative size");
    if (num_bin == 0) return GBX_OK;
    if (!A_glob || !E_glob || !A_template || !E_template || !start_ind || !group_index)
        return set_error(GBX_ERR_ARG, "NULL pointer");
    if (group_stride < data_length) return set_error(GBX_ERR_ARG, "group_stride < data_length");
    int rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    fill_global_kernel<<<grid_for(num_bin), 256, 0, (cudaStream_t)stream>>>(
        (double2 *)A_glob, (double2 *)E_glob, (const double2 *)A_template,
        (const double2 *)E_template, start_ind, M, num_bin, group_index, data_length,
        group_stride, t_stride_i, t_stride_b, num_groups, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "fill_global launch");
    return GBX_OK;
}

extern "C" int gbx_fill_global(void *A_glob, void *E_glob, const void *A_template,
                               const void *E_template, const int *start_ind, int M, int num_bin,
                               const int *group_index, int data_length, int *status, void *stream)
{
    return gbx_fill_global_ex(A_glob, E_glob, A_template, E_template, start_ind, M, num_bin,
                              group_index, data_length, 0, (long long)data_length,
                              (long long)num_bin, 1LL, status, stream);
}

extern "C" int gbx_fill_global_det(void *A_glob, void *E_glob, const void *A_template,
                                   const void *E_template, const int *start_ind, int M,
                                   int num_bin, const int *order, const int *group_first,
                                   int num_groups, int data_length, long long group_stride,
                                   long long t_stride_i, long long t_stride_b, void *stream)
{
    if (num_bin < 0 || M < 0 || data_length < 0 || num_groups < 0)
        return set_error(GBX_ERR_ARG, "negative size");
    if (num_groups == 0 || data_length == 0) return GBX_OK;
    if (!A_glob || !E_glob || !group_first || (num_bin > 0 && (!A_template || !E_template ||
                                                                !start_ind || !order)))
        return set_error(GBX_ERR_ARG, "NULL pointer");
    if (group_stride < data_length) return set_error(GBX_ERR_ARG, "group_stride < data_length");
    if (num_groups > 65535) return set_error(GBX_ERR_UNSUPPORTED, "at most 65535 groups");
    int rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    dim3 grid((data_length + kDetChunk - 1) / kDetChunk, num_groups);
    fill_det_kernel<<<grid, kDetThreads, 0, (cudaStream_t)stream>>>(
        (double2 *)A_glob, (double2 *)E_glob, (const double2 *)A_template,
        (const double2 *)E_template, start_ind, M, order, group_first, data_length, group_stride,
        t_stride_i, t_stride_b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "fill_det launch");
    return GBX_OK;
}
