// Drop-in replacements for the reference's two native kernels
// (gbgpu/cutils/gbgpu_utils.cu): batched <d|h>, <h|h> over point-major
// templates, and the scatter-add of templates into global buffers.
// get_ll: one warp per two binaries (lanes interleaved by binary); fill: one
// warp per binary, lanes along the window.
#include "gbx_common.cuh"
#include "gbx_internal.h"

namespace gbx {

// Re conj(d) h, Im conj(d) h and |h|^2 of one bin of one channel, before the
// PSD weight (float pairs, unnormalised sums: a tail stays below 2^-23 of the
// largest product, so a later product keeps ~1e-14 of sum |terms|)
__device__ __forceinline__ void ll_terms(double2 d, double2 hv, int eD, dfl &re, dfl &im, dfl &sq)
{
    const dfl dR = d2ff_scaled(d.x, eD), dI = d2ff_scaled(d.y, eD);
    const dfl hR = d2ff_scaled(hv.x, eD), hI = d2ff_scaled(hv.y, eD);
    re = df_sum(df_prod(dR, hR), df_prod(dI, hI));
    im = df_sum(df_prod(dR, hI), df_neg(df_prod(dI, hR)));
    sq = df_sum(df_prod(hR, hR), df_prod(hI, hI));
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
// FP64: the same mapping with the reference's arithmetic, FP64 products and
// sums (gbgpu_utils.cu:167-179, the division by S as a product with 1/S).
template <bool FP64>
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
        double xr = 0.0, xi = 0.0, xh = 0.0;
        bool out = false;
        const int Mh = use ? M : 0;
        // one PSD array for both channels (the usual call): one weight per bin
        const bool same = A_p == E_p;
        if constexpr (FP64) {
            for (int i = q; i < Mh; i += 16) {
                const int j = s + i;
                if (j < 0 || j >= L) {
                    out = true;
                    continue;
                }
                const double2 hA = __ldg(A_t + i * tsi + b * tsb);
                const double2 hE = __ldg(E_t + i * tsi + b * tsb);
                const double2 dA = __ldg(A_d + doff + j), dE = __ldg(E_d + doff + j);
                const double wA = 1.0 / __ldg(A_p + noff + j);
                const double wE = same ? wA : 1.0 / __ldg(E_p + noff + j);
                xr += (dA.x * hA.x + dA.y * hA.y) * wA + (dE.x * hE.x + dE.y * hE.y) * wE;
                xi += (dA.x * hA.y - dA.y * hA.x) * wA + (dE.x * hE.y - dE.y * hE.x) * wE;
                xh += (hA.x * hA.x + hA.y * hA.y) * wA + (hE.x * hE.x + hE.y * hE.y) * wE;
            }
        }
#pragma unroll 2
        for (int i = q; i < (FP64 ? 0 : Mh); i += 16) {
            const int j = s + i;
            if (j < 0 || j >= L) {
                out = true;
                continue;
            }
            const double2 hA = __ldg(A_t + i * tsi + b * tsb);
            const double2 hE = __ldg(E_t + i * tsi + b * tsb);
            const double2 dA = __ldg(A_d + doff + j), dE = __ldg(E_d + doff + j);
            dfl reA, imA, sqA, reE, imE, sqE;
            ll_terms(dA, hA, eD, reA, imA, sqA);
            ll_terms(dE, hE, eD, reE, imE, sqE);
            // accumulators stay normalised
            if (same) {
                const dfl w = df_recip(d2ff_scaled(__ldg(A_p + noff + j), eS));
                dr = df_add(dr, df_prod(df_sum(reA, reE), w));
                di = df_add(di, df_prod(df_sum(imA, imE), w));
                hh = df_add(hh, df_prod(df_sum(sqA, sqE), w));
            } else {
                const dfl wA = df_recip(d2ff_scaled(__ldg(A_p + noff + j), eS));
                const dfl wE = df_recip(d2ff_scaled(__ldg(E_p + noff + j), eS));
                dr = df_add(dr, df_sum(df_prod(reA, wA), df_prod(reE, wE)));
                di = df_add(di, df_sum(df_prod(imA, wA), df_prod(imE, wE)));
                hh = df_add(hh, df_sum(df_prod(sqA, wA), df_prod(sqE, wE)));
            }
        }
        if constexpr (FP64) {
#pragma unroll
            for (int o = 16; o > 1; o >>= 1) {
                xr += __shfl_xor_sync(0xffffffffu, xr, o);
                xi += __shfl_xor_sync(0xffffffffu, xi, o);
                xh += __shfl_xor_sync(0xffffffffu, xh, o);
            }
        } else {
            dr = pair_sum_df(dr);
            di = pair_sum_df(di);
            hh = pair_sum_df(hh);
        }
        if (__any_sync(0xffffffffu, out) && lane == 0) flag(status, GBX_FLAG_WINDOW);
        if (q == 0 && has) {
            if constexpr (FP64) {
                d_h[b] = make_double2(4. * df * xr, 4. * df * xi);
                h_h[b] = make_double2(4. * df * xh, 0.0);
            } else {
                // undo the scalings: terms carry 2^(2 eD - eS)
                const double s4 = 4. * df * __hiloint2double((eS - 2 * eD + 1023) << 20, 0);
                d_h[b] = make_double2(s4 * ((double)dr.h + (double)dr.l),
                                      s4 * ((double)di.h + (double)di.l));
                h_h[b] = make_double2(s4 * ((double)hh.h + (double)hh.l), 0.0);
            }
        }
    }
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

// Point-major templates (t_stride_b == 1, the reference's i * num_bin + b):
// one CTA per chunk of 32 binaries.  Slabs of 32 samples x 32 binaries are
// read one row per warp instruction (512 contiguous bytes), transposed
// through shared memory, and each warp then adds one binary's 32 consecutive
// bins with one reduction per lane and component, so the loads and the L2
// reductions of a warp instruction both cover contiguous addresses.  (One
// warp per binary on point-major rows reads 16 bytes per lane at a stride of
// num_bin x 16 bytes: half of every sector, and a long dependent chain.)
constexpr int kFillRows = 32;

__global__ void __launch_bounds__(256) fill_global_pm_kernel(
    double2 *__restrict__ A_g, double2 *__restrict__ E_g, const double2 *__restrict__ A_t,
    const double2 *__restrict__ E_t, const int *__restrict__ start_ind, int M, int num_bin,
    const int *__restrict__ group_index, int L, long long gstride, long long tsi, int num_groups,
    int *status)
{
    __shared__ double2 tA[kFillRows][33], tE[kFillRows][33];
    __shared__ long long s_goff[32];
    __shared__ int s_start[32], s_ok[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunks = (num_bin + 31) >> 5;
    for (int c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const int b0 = c << 5;
        if (threadIdx.x < 32) {
            const int b = b0 + threadIdx.x;
            int ok = 0, s = 0;
            long long goff = 0;
            if (b < num_bin) {
                s = start_ind[b];
                const int g = group_index[b];
                if (num_groups > 0 && (g < 0 || g >= num_groups)) {
                    flag(status, GBX_FLAG_INDEX);
                } else {
                    ok = 1;
                    goff = (long long)g * gstride;
                }
            }
            s_start[threadIdx.x] = s;
            s_goff[threadIdx.x] = goff;
            s_ok[threadIdx.x] = ok;
        }
        for (int i0 = 0; i0 < M; i0 += kFillRows) {
            __syncthreads();
            const int b = b0 + lane;
#pragma unroll
            for (int r = warp; r < kFillRows; r += 8) {
                const int i = i0 + r;
                double2 a = make_double2(0.0, 0.0), e = make_double2(0.0, 0.0);
                if (i < M && b < num_bin) {
                    a = __ldg(A_t + (size_t)i * tsi + b);
                    e = __ldg(E_t + (size_t)i * tsi + b);
                }
                tA[r][lane] = a;
                tE[r][lane] = e;
            }
            __syncthreads();
#pragma unroll
            for (int q = warp; q < 32; q += 8) {
                const int i = i0 + lane;
                const int j = s_start[q] + i;
                // gbgpu_utils.cu:88-91: bins outside the data are skipped
                if (!s_ok[q] || i >= M || j < 0 || j >= L) continue;
                const double2 a = tA[lane][q], e = tE[lane][q];
                const size_t o = (size_t)(s_goff[q] + j);
                atomicAdd(&A_g[o].x, a.x);
                atomicAdd(&A_g[o].y, a.y);
                atomicAdd(&E_g[o].x, e.x);
                atomicAdd(&E_g[o].y, e.y);
            }
        }
        __syncthreads();
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

template <bool FP64>
static int get_ll_launch(void *d_h, void *h_h, const void *A_template, const void *E_template,
                         const void *A_data, const void *E_data, const double *A_psd,
                         const double *E_psd, double df, const int *start_ind, int M, int num_bin,
                         const int *data_index, const int *noise_index, int data_length,
                         long long t_stride_i, long long t_stride_b, int num_data, int num_psd,
                         int *status, void *stream)
{
    if (num_bin < 0 || M < 0 || data_length < 0) return set_error(GBX_ERR_ARG, "negative size");
    if (num_bin == 0) return GBX_OK;
    if (!d_h || !h_h || !A_template || !E_template || !A_data || !E_data || !A_psd || !E_psd ||
        !start_ind)
        return set_error(GBX_ERR_ARG, "NULL pointer");
    int rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    get_ll_kernel<FP64><<<grid_for((num_bin + 1) / 2), 256, 0, (cudaStream_t)stream>>>(
        (double2 *)d_h, (double2 *)h_h, (const double2 *)A_template, (const double2 *)E_template,
        (const double2 *)A_data, (const double2 *)E_data, A_psd, E_psd, df, start_ind, M, num_bin,
        data_index, noise_index, data_length, t_stride_i, t_stride_b, num_data, num_psd, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "get_ll launch");
    return GBX_OK;
}

extern "C" int gbx_get_ll_ex(void *d_h, void *h_h, const void *A_template,
                             const void *E_template, const void *A_data, const void *E_data,
                             const double *A_psd, const double *E_psd, double df,
                             const int *start_ind, int M, int num_bin, const int *data_index,
                             const int *noise_index, int data_length, long long t_stride_i,
                             long long t_stride_b, int num_data, int num_psd, int *status,
                             void *stream)
{
    return get_ll_launch<false>(d_h, h_h, A_template, E_template, A_data, E_data, A_psd, E_psd,
                                df, start_ind, M, num_bin, data_index, noise_index, data_length,
                                t_stride_i, t_stride_b, num_data, num_psd, status, stream);
}

extern "C" int gbx_get_ll_fp64(void *d_h, void *h_h, const void *A_template,
                               const void *E_template, const void *A_data, const void *E_data,
                               const double *A_psd, const double *E_psd, double df,
                               const int *start_ind, int M, int num_bin, const int *data_index,
                               const int *noise_index, int data_length, long long t_stride_i,
                               long long t_stride_b, int num_data, int num_psd, int *status,
                               void *stream)
{
    return get_ll_launch<true>(d_h, h_h, A_template, E_template, A_data, E_data, A_psd, E_psd,
                               df, start_ind, M, num_bin, data_index, noise_index, data_length,
                               t_stride_i, t_stride_b, num_data, num_psd, status, stream);
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
    if (t_stride_b == 1 && t_stride_i >= num_bin) {
        // point-major templates: coalesced slabs through shared memory
        const int chunks = (num_bin + 31) / 32;
        const int cap = num_sms() * 6;
        fill_global_pm_kernel<<<chunks < cap ? chunks : cap, 256, 0, (cudaStream_t)stream>>>(
            (double2 *)A_glob, (double2 *)E_glob, (const double2 *)A_template,
            (const double2 *)E_template, start_ind, M, num_bin, group_index, data_length,
            group_stride, t_stride_i, num_groups, status);
    } else {
        fill_global_kernel<<<grid_for(num_bin), 256, 0, (cudaStream_t)stream>>>(
            (double2 *)A_glob, (double2 *)E_glob, (const double2 *)A_template,
            (const double2 *)E_template, start_ind, M, num_bin, group_index, data_length,
            group_stride, t_stride_i, t_stride_b, num_groups, status);
    }
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
