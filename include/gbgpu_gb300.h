/*
 * gbgpu_gb300 -- C ABI of the GB300 (sm_103a) FastGB hot path.
 *
 * Every entry point takes caller-owned DEVICE pointers, plain sizes and a
 * CUDA stream handle (cudaStream_t passed as void*, NULL = legacy default
 * stream), launches asynchronously on that stream and returns a status code
 * (GBX_OK = 0).  The library works in the CUDA runtime's context of the
 * current device (its primary context): its per-device set-up (FFT tables,
 * the allocation-free scratch address) is done once per device in that
 * context, so making another context current is not supported.  Nothing is allocated per call, nothing is synchronised, and
 * no call ever terminates the process (the reference's gpuAssert calls
 * exit(), gbgpu/cutils/global.h:46-54).  Complex arrays are interleaved
 * double[2] (complex128), the layout of the reference's
 * gcmplx::complex<double> (gbgpu/cutils/global.h:66).
 */
#ifndef GBGPU_GB300_H
#define GBGPU_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes returned by every entry point ---- */
#define GBX_OK 0
#define GBX_ERR_ARG 1          /* NULL pointer, negative size, bad index array ... */
#define GBX_ERR_UNSUPPORTED 2  /* N not a power of two or outside the supported range */
#define GBX_ERR_CUDA 3         /* the CUDA runtime reported an error (see gbx_last_error) */

/* ---- bits OR-ed by kernels into the optional device status word ---- */
#define GBX_FLAG_WINDOW 1      /* a template window left [0, data_length): those bins count as 0 */
#define GBX_FLAG_INDEX 2       /* a data_index / noise_index / group_index out of range: binary skipped */
#define GBX_FLAG_TILE 4        /* malformed tile descriptor: tile skipped */

/* ---- precision of the waveform family ---- */
#define GBX_FP64 0             /* every step in FP64 (the plain form) */
#define GBX_MIXED 1            /* FP64 carrier phase, delays and reductions; FP32 slow part + FFT */
#define GBX_PAIR 2             /* slow part, FFT and <d|h> in float pairs (FP32 pipe, ~44 bits);
                                  waveform, likelihood, fill and swap entry points,
                                  9 parameters, N <= 4096 */

#define GBX_MAX_LOG2N 13       /* N = 2^k, 5 <= k <= 13 (FP64 form: k <= 12) */

/* ---- bits of gbx_wave_args.tdi2 ---- */
#define GBX_TDI2_BIT 1         /* second-generation TDI */
#define GBX_TDI_UNEQUAL 2      /* per-sample arm lengths |P_j - P_i| (no counterpart in the reference) */

int gbx_version(void);

/* Message for the most recent non-zero status returned on this host thread. */
const char *gbx_last_error(void);

/* Number of SMs and compute capability (major*10 + minor) of the current device. */
int gbx_device_info(int *num_sms, int *arch);

/*
 * One-time set-up on the current device (FFT twiddle tables).  Every entry
 * point does it on first use and synchronises its stream once to do so; call
 * gbx_init() first when the first call would otherwise be made while a
 * stream is being captured into a CUDA graph.
 */
int gbx_init(void);

/*
 * Drop-in for get_ll_wrap (reference: gbgpu/cutils/gbgpu_utils.hh:11-13,
 * kernel gbgpu/cutils/gbgpu_utils.cu:124-210).  Same argument order and
 * meaning: for each binary b,
 *   d_h[b] = 4 df sum_{i<M} sum_{A,E} conj(d[di*L + s_b + i]) h[i*num_bin + b] / S[ni*L + s_b + i]
 *   h_h[b] = 4 df sum_{i<M} sum_{A,E} |h[i*num_bin + b]|^2 / S[ni*L + s_b + i]
 * with templates in the reference's point-major layout (element i*num_bin+b).
 * Differences: bins outside [0, data_length) contribute zero and set
 * GBX_FLAG_WINDOW in *status (the reference reads out of bounds); the call is
 * asynchronous on `stream` (the reference synchronises the device); the
 * products and sums run in float-pair arithmetic (46 significant bits per
 * input), so each output is within 1e-12 of sum |terms| of the FP64 sums
 * (the reference sums in FP64); a PSD bin at infinity contributes zero.
 * data_index / noise_index may be NULL (row 0 for every binary).  The
 * reference's argument list carries no row counts, so only negative rows are
 * rejected here (flagged GBX_FLAG_INDEX, not read, zero outputs); the caller
 * keeps di*L and ni*L inside its data and PSD arrays, or calls gbx_get_ll_ex
 * with the row counts.  `status` may be NULL.
 */
int gbx_get_ll(void *d_h, void *h_h, const void *A_template, const void *E_template,
               const void *A_data, const void *E_data, const double *A_psd,
               const double *E_psd, double df, const int *start_ind, int M,
               int num_bin, const int *data_index, const int *noise_index,
               int data_length, int *status, void *stream);

/*
 * gbx_get_ll with explicit template strides: element (b, i) of a template is
 * read at A_template[i * t_stride_i + b * t_stride_b] (in complex elements).
 * (num_bin, 1) is the reference's point-major layout; (1, M) reads a
 * (num_bin, M) row-major array without the transpose the reference makes.
 * num_data / num_psd > 0 are the rows of the data and PSD arrays: a binary
 * whose data_index / noise_index lies outside them is flagged GBX_FLAG_INDEX,
 * not read, and gets zero outputs (0 = rows not known; negative rows are
 * always rejected).
 */
int gbx_get_ll_ex(void *d_h, void *h_h, const void *A_template, const void *E_template,
                  const void *A_data, const void *E_data, const double *A_psd,
                  const double *E_psd, double df, const int *start_ind, int M, int num_bin,
                  const int *data_index, const int *noise_index, int data_length,
                  long long t_stride_i, long long t_stride_b, int num_data, int num_psd,
                  int *status, void *stream);

/*
 * gbx_get_ll_ex with the reference's arithmetic: FP64 products and sums
 * (gbgpu/cutils/gbgpu_utils.cu:167-179; the division by S as a product with
 * 1/S), for callers that want the FP64 result itself rather than one within
 * 1e-12 of sum |terms|.  Same arguments, edge rules and flags; 3x the time
 * of gbx_get_ll_ex on GB300 (0.63 against 0.21 ms for 50k windows of 256
 * bins), whose FP64 rate is 1/64 of its FP32 rate.
 */
int gbx_get_ll_fp64(void *d_h, void *h_h, const void *A_template, const void *E_template,
                    const void *A_data, const void *E_data, const double *A_psd,
                    const double *E_psd, double df, const int *start_ind, int M, int num_bin,
                    const int *data_index, const int *noise_index, int data_length,
                    long long t_stride_i, long long t_stride_b, int num_data, int num_psd,
                    int *status, void *stream);

/*
 * Drop-in for fill_global_wrap (reference: gbgpu/cutils/gbgpu_utils.hh:6-7,
 * kernel gbgpu/cutils/gbgpu_utils.cu:54-122):
 *   glob[group_index[b]*L + start_ind[b] + i] += template[i*num_bin + b]
 * for 0 <= start_ind[b] + i < data_length, channels A and E, accumulated with
 * native FP64 atomics (the reference emulates them with a CAS loop).
 */
int gbx_fill_global(void *A_glob, void *E_glob, const void *A_template,
                    const void *E_template, const int *start_ind, int M, int num_bin,
                    const int *group_index, int data_length, int *status, void *stream);

/*
 * gbx_fill_global with strides: group g of a channel starts at element
 * g * group_stride (>= data_length), so channels 0 and 1 of a caller's
 * (G, nch, L) template array are filled in place with group_stride = nch*L --
 * the reference instead fills two G*L temporaries and copies them back
 * (gbgpu/gbgpu.py:796-837).  Template strides as in gbx_get_ll_ex.  When
 * num_groups > 0, group indices outside [0, num_groups) are skipped and
 * flagged with GBX_FLAG_INDEX.
 */
int gbx_fill_global_ex(void *A_glob, void *E_glob, const void *A_template,
                       const void *E_template, const int *start_ind, int M, int num_bin,
                       const int *group_index, int data_length, int num_groups,
                       long long group_stride, long long t_stride_i, long long t_stride_b,
                       int *status, void *stream);

/*
 * Deterministic form of gbx_fill_global_ex (no counterpart in the reference,
 * whose GPU fill order depends on atomic scheduling).  `order` lists the
 * binaries sorted by (group, start index) and group_first[g] ..
 * group_first[g+1] is group g's slice of it (num_groups + 1 entries).  Every
 * bin of channels A/E of every group is written -- the sum of the windows that
 * reach it, added in `order`, or zero -- so repeated calls give identical
 * bits and the reference's overwrite semantics hold without zeroing first.
 * Group indices themselves are implied by group_first.
 */
int gbx_fill_global_det(void *A_glob, void *E_glob, const void *A_template,
                        const void *E_template, const int *start_ind, int M, int num_bin,
                        const int *order, const int *group_first, int num_groups,
                        int data_length, long long group_stride, long long t_stride_i,
                        long long t_stride_b, void *stream);

/*
 * Orbit table for one N.  `sc_pos` is the (3, N, 3) FP64 array of spacecraft
 * positions [m] at tm_n = n T/N for spacecraft 1, 2, 3 -- exactly what the
 * reference obtains from orbits.get_pos (gbgpu/gbgpu.py:390-397).  The table
 * holds P_s/c and the arm unit vectors r_12, r_23, r_31 = (P_j - P_i)/L
 * (gbgpu/gbgpu.py:424-427) in FP64 and FP32; it is what the waveform family
 * reads.  `table` must hold gbx_orbit_table_bytes(N) bytes, 16-byte aligned.
 * Layout (rows of N, sample n fastest): 18 FP64 rows P_s/c, r_12, r_23,
 * r_31; then 36 FP32 rows: r (9), P_s/c as float pairs (9 heads, 9 tails),
 * r's tails (9).
 */
size_t gbx_orbit_table_bytes(int N);
int gbx_orbit_table(void *table, const double *sc_pos, int N, double armlength,
                    void *stream);

/*
 * Batch description shared by the waveform family.  Parameters are a
 * (nparams, num_bin) row-major FP64 array -- the reference's `params` layout
 * for get_ll (gbgpu/gbgpu.py:597-599): amp, f0, fdot, fddot, phi0, iota, psi,
 * lam, beta, followed for the third-body model by A2, varpi, e2, P2 [yr],
 * T2 [yr] (gbgpu/thirdbody.py:39-80).
 *
 * Uniform N: set N and leave tiles NULL.  Uneven N: set N = 0 and pass a tile
 * list; tile t is four ints {log2 N, first slot, count, 0}; slots map to
 * binaries through `order` (NULL = identity) and count <= max(1, 512/N).
 * With `queue` non-NULL the tiles are taken from a device work-queue counter
 * (reset by the call, so concurrent calls must not share it); tiles should be
 * sorted by decreasing N for load balance.
 */
typedef struct gbx_wave_args {
    const double *params;
    int num_bin;
    int nparams;                 /* 9, or 14 for the third-body model */
    int N;                       /* uniform N (power of two) or 0 with tiles */
    int precision;               /* GBX_FP64, GBX_MIXED or GBX_PAIR */
    int tdi2;                    /* bit 0 (GBX_TDI2_BIT): TDI-2; bit 1 (GBX_TDI_UNEQUAL): unequal arms.
                                    0: TDI-1.5, 1: times 2i sin(2wL) e^{-2iwL} at f0 (the reference's
                                    equal-arm forms); 2, 3: per-sample arm lengths from the orbit
                                    table (FP64 and pair forms, 9 parameters; otherwise
                                    GBX_ERR_UNSUPPORTED) */
    int start_freq_ind;          /* subtracted from every start index */
    double T;                    /* observation time, already int(T/dt)*dt */
    double armlength;            /* m */
    double year;                 /* seconds per year used for P2, T2 (third body) */
    const void *orbit[GBX_MAX_LOG2N + 1];   /* table for N = 2^k, NULL if unused */
    const int *order;
    const int *tiles;
    int ntiles;
    int *queue;
    int *status;                 /* optional device word for GBX_FLAG_* bits */
    void *workspace;             /* optional scratch of gbx_wave_workspace_bytes(num_bin) */
    size_t workspace_bytes;
    /* Launch shape (0 = defaults).  tile: samples per tile, a power of two
     * in [64, 4096]; a tile holds clamp(tile / N, 1, 16) binaries of one N
     * (at least 2 for gbx_swap_ll) and the likelihood epilogue gives each
     * binary 256 / that many threads.  Default 512.  blocks_per_sm: resident
     * persistent blocks per SM, capped by occupancy; default as many as fit.
     * Tile lists passed in `tiles` must be packed with the same tile. */
    int tile;
    int blocks_per_sm;
} gbx_wave_args;

/*
 * Scratch for the per-binary constants of one call (16-byte aligned).  With a
 * workspace the constants are computed by a separate fully occupied kernel
 * before the waveform kernel; with workspace = NULL each tile computes them
 * itself (same results, slower for large batches).  Calls that run at the
 * same time must not share a workspace.
 */
size_t gbx_wave_workspace_bytes(int num_bin);

/* Data side of the likelihood: (num_data, L) complex128 data, (num_psd, L) PSD. */
typedef struct gbx_ll_args {
    const void *A_data;
    const void *E_data;
    const double *A_psd;
    const double *E_psd;
    int data_length;
    int num_data;
    int num_psd;
    const int *data_index;       /* NULL = all zeros */
    const int *noise_index;      /* NULL = all zeros */
    double df;
} gbx_ll_args;

/*
 * run_wave (reference gbgpu/gbgpu.py:108-316): X/Y/Z and A/E/T frequency-domain
 * windows as (num_bin, 3, N) complex128 (either output may be NULL) and the
 * start indices (int32, start_freq_ind subtracted).  Uniform N only.
 */
int gbx_waveform(const gbx_wave_args *a, void *XYZ_out, void *AET_out, int *start_out,
                 void *stream);

/*
 * Fused run_wave + get_ll (reference gbgpu/gbgpu.py:580-712 with the native
 * kernel gbgpu_utils.cu:124-185): d_h and h_h (complex128, num_bin) without
 * writing the waveform to memory.  Uniform or uneven N.
 */
int gbx_waveform_ll(const gbx_wave_args *a, const gbx_ll_args *l, void *d_h, void *h_h,
                    void *stream);

/*
 * Fused run_wave + fill_global (reference gbgpu/gbgpu.py:839-878): scatter-adds
 * A and E of every binary into A_glob/E_glob[group_index[b]*L + j] with FP64
 * atomics.  Group g starts at element g * group_stride (0 = data_length).
 * The caller zeroes the templates first when it wants the reference's
 * overwrite semantics (gbgpu/gbgpu.py:796-801, 836-837).
 */
int gbx_waveform_fill(const gbx_wave_args *a, void *A_glob, void *E_glob,
                      const int *group_index, int num_groups, int data_length,
                      long long group_stride, void *stream);

/*
 * Swap log-likelihood (no counterpart in this version of the reference; the
 * library's own definition): for each pair j, binaries 2j (the current source)
 * and 2j+1 (the proposal) of the batch, with r the residual row chosen by
 * data_index[2j+1] (d minus the walker's current sum of sources) and
 * Dh = h_new - h_old,
 *   dlogl[j] = Re<r|Dh> - 1/2 <Dh|Dh>
 * with <a|b> = 4 df sum_{A,E} conj(a) b / S over the union of both windows
 * (the inner product of gbgpu/cutils/gbgpu_utils.cu:172-183).  Uniform N,
 * num_bin even; FP64, pair and FP32 forms (the pair form for 9 parameters);
 * circular or third-body parameters.
 */
int gbx_swap_ll(const gbx_wave_args *a, const gbx_ll_args *l, double *dlogl, void *stream);

/*
 * Fused waveform + likelihood + gradient (no counterpart in the reference,
 * which has only finite-difference Fisher matrices, gbgpu/gbgpu.py:957-1138).
 * Computes d_h, h_h as gbx_waveform_ll and grad[k*num_bin + b] =
 * d logL_b / d params[k, b] for the nine parameters (amp, f0, fdot, fddot,
 * phi0, iota, psi, lam, beta) of logL = -1/2 (<d|d> + <h|h> - 2 Re<d|h>),
 * and with nparams = 14 also for the third body's (A2, varpi, e2, P2, T2).
 * Mixed form only (N <= 2048 for the third body).  The workspace is required
 * and must hold gbx_grad_workspace_bytes(num_bin) bytes.
 */
size_t gbx_grad_workspace_bytes(int num_bin);
int gbx_waveform_ll_grad(const gbx_wave_args *a, const gbx_ll_args *l, void *d_h, void *h_h,
                         double *grad, void *stream);

/*
 * Swap log-likelihood with its gradient (no counterpart in the reference):
 * the pairs, residual rows and dlogl of gbx_swap_ll (dlogl may be NULL), and
 * grad[k*(num_bin/2) + j] = d dlogl[j] / d params[k, 2j+1], the gradient with
 * respect to the proposal, = Re<r + h_old - h_new | d h_new / d theta>
 * (the likelihood gradient at the proposal against the data r + h_old).
 * Mixed form only, uniform N, num_bin even, 9 or 14 parameters; the workspace
 * must hold gbx_grad_workspace_bytes(num_bin) bytes.  Two launches: the swap
 * kernel for dlogl, then the gradient kernel with each tile's pairs.
 */
int gbx_swap_ll_grad(const gbx_wave_args *a, const gbx_ll_args *l, double *dlogl, double *grad,
                     void *stream);

/*
 * Per-binary Fisher matrices by forward mode in one launch (the reference
 * forms them from five-point differences of run_wave, gbgpu/gbgpu.py:957-1138):
 * fisher[b*81 + 9*i + j] = 4 df sum_{A,E} Re conj(dh/dp_i) dh/dp_j / S over the
 * binary's window, p = (amp, f0, fdot, fddot, phi0, iota, psi, lam, beta),
 * with S the PSD rows A_psd / E_psd (num_psd rows of psd_length bins, row
 * noise_index[b] or 0; bin j of a row is bin j + start_freq_ind of the grid).
 * Mixed form, 9 parameters, equal arms; the workspace must hold
 * gbx_grad_workspace_bytes(num_bin) bytes; tiles of at most 1024 samples.
 */
int gbx_fisher(const gbx_wave_args *a, const double *A_psd, const double *E_psd, int psd_length,
               int num_psd, const int *noise_index, double df, double *fisher, void *stream);

/*
 * gbx_waveform_ll without caller-provided scratch.  No counterpart in the
 * reference (its kernels use no scratch).  For callers that may not allocate
 * device memory: a plug-in inside an application that owns all device
 * allocations, or an FFI binding with no CUDA allocator.  The per-binary
 * workspace and the work-queue counter live in one static device array of
 * GBX_NOALLOC_MAX_BINS * 512 + 256 bytes (4 MiB) that every GPU loading the
 * library keeps until the process exits; a->workspace and a->queue are
 * ignored.  Batches above GBX_NOALLOC_MAX_BINS binaries are rejected with
 * GBX_ERR_ARG.  Nothing is allocated: no cudaMalloc/cudaFree or allocating
 * library call.  The first call on a device looks up the array's device
 * address (and, like every entry point, builds the FFT tables and
 * synchronises its stream once); make that first call before any stream
 * capture.  All calls share the array: calls whose kernels overlap on the GPU
 * (different streams, or different host threads) race on it and must be
 * serialised by the caller.  The counter is cleared on the stream before
 * each launch; the workspace is fully rewritten by every call.  The caller
 * still provides its inputs, outputs, orbit tables and (uneven N) tile and
 * order lists as device memory of its own.
 */
#define GBX_NOALLOC_MAX_BINS 8192
int gbx_waveform_ll_noalloc(const gbx_wave_args *a, const gbx_ll_args *l, void *d_h,
                            void *h_h, void *stream);

/*
 * Diagnostic: evaluates one of the kernels' own math helpers on n device
 * inputs x (no counterpart in the reference), for tests against FP64 or a
 * host restatement.  which = 0: x is float, out[2i], out[2i+1] = sin(x[i]),
 * cos(x[i]) by the helper the mixed kernels use for reduced phases and
 * omega L; which = 1: x is float, sin(a)/a and cos(a) of the link transfer
 * functions; which = 2: x is double, out[i] = x[i] * 2^e rounded to FP32 by
 * the integer-pipe conversion of the mixed likelihood.
 */
int gbx_math_selftest(const void *x, float *out, int n, int which, int e, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GBGPU_GB300_H */
