// C ABI plumbing: error reporting, one-time device set-up, orbit tables.
#include <mutex>
#include <stdarg.h>
#include <stdio.h>

#include "gbx_common.cuh"
#include "gbx_internal.h"

static thread_local char g_msg[512] = "";

int set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_error(cudaError_t e, const char *what)
{
    return set_error(GBX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

namespace {
constexpr int kMaxDev = 64;
std::mutex g_lock;
bool g_ready[kMaxDev] = {};
int g_sms[kMaxDev] = {};
}  // namespace

int num_sms()
{
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDev) return 1;
    if (g_sms[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        g_sms[dev] = n > 0 ? n : 1;
    }
    return g_sms[dev];
}

// Per-device one-time set-up (the FFT twiddle tables in __device__ memory).
// It synchronises the given stream once, so the first call on a device must
// not happen while that stream is being captured into a CUDA graph.
int ensure_init(cudaStream_t st)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDev) return set_error(GBX_ERR_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> g(g_lock);
    if (g_ready[dev]) return GBX_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    if (cs != cudaStreamCaptureStatusNone)
        return set_error(GBX_ERR_ARG, "first call on a device inside stream capture: call gbx_init() first");
    int rc = gbx_twiddle_init(st);
    if (rc) return rc;
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "twiddle init sync");
    g_ready[dev] = true;
    num_sms();
    return GBX_OK;
}

extern "C" int gbx_version(void) { return 100; }

extern "C" const char *gbx_last_error(void) { return g_msg; }

extern "C" int gbx_init(void) { return ensure_init(0); }

extern "C" int gbx_device_info(int *num_sms_out, int *arch)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    int maj = 0, mnr = 0;
    cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&mnr, cudaDevAttrComputeCapabilityMinor, dev);
    if (num_sms_out) *num_sms_out = num_sms();
    if (arch) *arch = maj * 10 + mnr;
    return GBX_OK;
}

// ---------------------------------------------------------------- orbit table
// double rows (3s+c)*N + n : P_s[c]/c ;  rows (9 + 3a + c)*N + n : r_a[c]
// float  rows (3a+c)*N + n : r_a[c]    (a = 12, 23, 31)
//        rows (9 + 3s + c)*N + n, (18 + 3s + c)*N + n : P_s[c]/c as a float pair hi, lo
//        rows (27 + 3a + c)*N + n : r_a[c] - (float)r_a[c] (the pair form's tails)
__global__ void orbit_table_kernel(double *tab, const double *pos, int N, double L)
{
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float *tf = reinterpret_cast<float *>(tab + (size_t)18 * N);
    double P[3][3];
    for (int s = 0; s < 3; s++)
        for (int c = 0; c < 3; c++) P[s][c] = pos[((size_t)s * N + n) * 3 + c];
    for (int s = 0; s < 3; s++)
        for (int c = 0; c < 3; c++) {
            double pc = P[s][c] / gbx::kCSI;
            float hi = (float)pc;
            tab[(size_t)(3 * s + c) * N + n] = pc;
            tf[(size_t)(9 + 3 * s + c) * N + n] = hi;
            tf[(size_t)(18 + 3 * s + c) * N + n] = (float)(pc - (double)hi);
        }
    for (int c = 0; c < 3; c++) {
        // gbgpu.py:424-427: r12 = (P2 - P1)/L, r23 = (P3 - P2)/L, r31 = -(P3 - P1)/L
        double r12 = (P[1][c] - P[0][c]) / L;
        double r23 = (P[2][c] - P[1][c]) / L;
        double r31 = -((P[2][c] - P[0][c]) / L);
        tab[(size_t)(9 + c) * N + n] = r12;
        tab[(size_t)(12 + c) * N + n] = r23;
        tab[(size_t)(15 + c) * N + n] = r31;
        const double rr[3] = {r12, r23, r31};
        for (int a = 0; a < 3; a++) {
            const float hi = (float)rr[a];
            tf[(size_t)(3 * a + c) * N + n] = hi;
            tf[(size_t)(27 + 3 * a + c) * N + n] = (float)(rr[a] - (double)hi);
        }
    }
}

extern "C" size_t gbx_orbit_table_bytes(int N)
{
    if (N <= 0) return 0;
    return (size_t)N * (18 * sizeof(double) + 36 * sizeof(float));
}

extern "C" int gbx_orbit_table(void *table, const double *sc_pos, int N, double armlength,
                               void *stream)
{
    if (!table || !sc_pos) return set_error(GBX_ERR_ARG, "NULL orbit pointer");
    if (N < 32 || (N & (N - 1)) != 0 || N > (1 << GBX_MAX_LOG2N))
        return set_error(GBX_ERR_UNSUPPORTED, "orbit table N=%d", N);
    if (!(armlength > 0.0)) return set_error(GBX_ERR_ARG, "armlength must be > 0");
    if (((uintptr_t)table & 15) != 0) return set_error(GBX_ERR_ARG, "table must be 16-byte aligned");
    orbit_table_kernel<<<(N + 127) / 128, 128, 0, (cudaStream_t)stream>>>((double *)table, sc_pos, N,
                                                                         armlength);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "orbit table launch");
    return GBX_OK;
}
