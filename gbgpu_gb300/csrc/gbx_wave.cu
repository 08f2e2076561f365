// FastGB waveform family for GB300 (sm_103a): one CTA builds a tile of
// binaries (P = max(1, 512/N) of them) entirely in shared memory -- slow part,
// N-point FFT, fftshift/heterodyne and TDI combination -- and then either
// writes the reference's output arrays, folds the window into <d|h>, <h|h>
// against the data and PSD, or scatter-adds it into global templates.
//
// Reference: gbgpu/gbgpu.py:108-578 (waveform), gbgpu/thirdbody.py:155-428
// (third body), gbgpu/cutils/gbgpu_utils.cu:54-185 (likelihood / fill loops).
#include <math.h>
#include <string.h>

#include <mutex>
#include <type_traits>

#include "gbx_common.cuh"
#include "gbx_internal.h"

extern "C" size_t gbx_wave_workspace_bytes(int num_bin);

namespace gbx {

__device__ double2 g_tw_d[kTwN / 2];
__device__ float2 g_tw_f[kTwN / 2];
__device__ float4 g_tw_p[kTwN / 2];   // the same twiddles as float pairs (c.h, c.l, s.h, s.l)
__device__ float4 g_sc_p[256];        // cos, sin of j pi/128 as float pairs (pair form)

__global__ void tw_init_kernel()
{
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < kTwN / 2) {
        double s, c;
        sincospi(-2.0 * (double)m / (double)kTwN, &s, &c);
        g_tw_d[m] = make_double2(c, s);
        g_tw_f[m] = make_float2((float)c, (float)s);
        const dfl cp = df_from(c), sp = df_from(s);
        g_tw_p[m] = make_float4(cp.h, cp.l, sp.h, sp.l);
    }
    if (m < 256) {
        double s, c;
        sincospi((double)m / 128.0, &s, &c);
        const dfl cp = df_from(c), sp = df_from(s);
        g_sc_p[m] = make_float4(cp.h, cp.l, sp.h, sp.l);
    }
}

template <typename R> __device__ __forceinline__ typename C2<R>::T tw(int m);
template <> __device__ __forceinline__ float2 tw<float>(int m) { return g_tw_f[m]; }
template <> __device__ __forceinline__ double2 tw<double>(int m) { return g_tw_d[m]; }

// ----------------------------------------------------------------------------
// per-binary constants (shared memory)
// ----------------------------------------------------------------------------
struct __align__(16) Bin {
    double f0, fdot, fddot, phi0;
    double om, om_m_dfa;           // 2 pi f0, 2 pi f0 - 2 pi q/T   (gbgpu.py:462-464)
    double pifdot, pi3fddot;       // pi fdot, pi/3 fddot           (gbgpu.py:495-500)
    double k[3];
    union {
        struct {
            double ep[6], ec[6];   // e+ and ex, order xx yy zz xy xz yz (FP64 form)
        } q;
        struct {
            dfl ud[3], vd[2];      // u and v (v has no z component) as pairs (pair form)
            cpx DP, DC;            // polarisation factors divided by amp, as pairs
        } pr;
    };
    double2 DP, DC;                // polarisation factors divided by amp
    double2 scale;                 // amp * 0.5 T / N [* tdi2 factor]
    double A2, varpi, e2;          // third body (FP64 form)
    union { double n2; dfl n2d; }; // n2 [rad/s]: FP64 form / float pair (mixed form)
    union { double T2; dfl T2d; }; // T2 [s], likewise
    float kf[3], uf[3], vf[3];      // k, u, v in FP32 (mixed form; r.e+.r = (r.v)^2 - (r.u)^2)
    float2 DPf, DCf;
    float f0f, fdotf, fddotf;
    float w0h, w0l, w1, w2;        // f(t)/fstar = (w0h + w0l) + w1 t + w2 t^2 (w0 split hi/lo)
    float w1l;                     // w1 - (float)w1 (the pair form's w1 t term)
    dfl kd[3], omd, omdfad, phi0d, pfd;   // float-pair copies for the mixed carrier phase
    dfl tpfd;                      // 2 pi fdot as a float pair
    dfl p3d, pfddd;                // pi/3 fddot, pi fddot (the mixed form uses the heads)
    float A2f, e2f, varpif, sinvarpif;
    int start;                     // start index - start_freq_ind
    int b;                         // binary index
    int di, ni, gi;                // data / noise / group rows
    int eS, eD;                    // power-of-two scalings of the mixed likelihood
    int valid;
};

static_assert(sizeof(Bin) % 16 == 0, "Bin is copied as int4 vectors");

struct KParams {
    gbx_wave_args a;
    // likelihood
    const double2 *A_data, *E_data;
    const double *A_psd, *E_psd;
    int L, num_data, num_psd;
    const int *data_index, *noise_index;
    double df;
    double2 *d_h, *h_h;
    double *dlogl;                 // swap: one log-likelihood change per (old, new) pair
    // waveform outputs
    double2 *XYZ, *AET;
    int *start_out;
    // fill
    double2 *A_glob, *E_glob;
    const int *group_index;
    int num_groups;
    long long gstride;             // elements between consecutive groups of A_glob / E_glob
    int P;                         // binaries per tile in uniform mode
    double fstar;                  // c / (2 pi L)
    dfl stepd[GBX_MAX_LOG2N + 1];  // T / 2^k as float pairs (exact: division by a power of two)
    dfl Locd;                      // L / c as a float pair (pair form)
    int maxS;                      // largest tile (samples) the shared memory is sized for
    int maxP;                      // most binaries in a tile of this launch (<= kMaxPack)
};

enum { MODE_WAVE = 0, MODE_LL = 1, MODE_FILL = 2, MODE_SWAP = 4 };

// doubles of the per-tile reduction scratch: 3 per 32-sample chunk, and at
// least 8 per lane group (16 groups) for the swap epilogue
// group partials of the likelihood (up to kMaxPack groups x 3 float pairs) and
// the per-binary FP64 sums (up to kMaxPack x 3) after them, or the swap
// epilogue's group x 8 FP64 partials
__host__ __device__ __forceinline__ int red_doubles(int maxS)
{
    return 3 * (maxS >> 5) > 8 * kMaxPack ? 3 * (maxS >> 5) : 8 * kMaxPack;
}

__device__ __forceinline__ double quad_form(const double *e, double x, double y, double z)
{
    return e[0] * x * x + e[1] * y * y + e[2] * z * z +
           2.0 * (e[3] * x * y + e[4] * x * z + e[5] * y * z);
}

// sin(x) and cos(x) for moderate |x| (the carrier phase reduced to [-pi, pi],
// omega L, link arguments: |x| < 8).  Cody-Waite reduction r = x - k pi/2
// with pi/2 split into two floats (Cody & Waite, "Software Manual for the
// Elementary Functions", 1980), then the Taylor series of sin and cos on
// |r| <= pi/4 (truncation below 2e-9 and 2e-10), then the quadrant k mod 4.
__device__ __forceinline__ void sincos_mod(float x, float &s, float &c)
{
    constexpr float kTwoOverPi = 0.636619772367581343f;
    constexpr float kPio2Hi = 1.57079637050628662f;       // float(pi/2)
    constexpr float kPio2Lo = -4.37113900018624283e-8f;   // pi/2 - float(pi/2)
    const float k = rintf(x * kTwoOverPi);
    const float r = fmaf(-k, kPio2Lo, fmaf(-k, kPio2Hi, x));
    const float r2 = r * r;
    float ps = fmaf(r2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = fmaf(r2, ps, 1.0f / 120.0f);
    ps = fmaf(r2, ps, -1.0f / 6.0f);
    const float sr = fmaf(r * r2, ps, r);
    float pc = fmaf(r2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = fmaf(r2, pc, -1.0f / 720.0f);
    pc = fmaf(r2, pc, 1.0f / 24.0f);
    pc = fmaf(r2, pc, -0.5f);
    const float cr = fmaf(r2, pc, 1.0f);
    const int q = (int)k;
    const float a = (q & 1) ? cr : sr, b = (q & 1) ? sr : cr;
    s = (q & 2) ? -a : a;
    c = ((q + 1) & 2) ? -b : b;
}

// sin(a)/a and cos(a) from their Taylor series in x = a^2: 3 and 4 terms for
// |a| < 0.16 (truncation below 4e-9 and 1e-11), 4 and 5 terms for |a| < 0.5
// (below 3e-8 and 3e-10), 8 terms up to |a| = 1.6 (below 2e-10); sincos_mod
// beyond that.
__device__ __forceinline__ void sinc_cos_f(float a, float &S, float &C)
{
    const float x = a * a;
    if (x < 0.0256f) {
        S = fmaf(fmaf(x, 1.0f / 120.0f, -1.0f / 6.0f), x, 1.0f);
        float c = fmaf(x, -1.0f / 720.0f, 1.0f / 24.0f);
        c = fmaf(c, x, -0.5f);
        C = fmaf(c, x, 1.0f);
    } else if (x < 0.25f) {
        float s = fmaf(x, -1.0f / 5040.0f, 1.0f / 120.0f);
        s = fmaf(s, x, -1.0f / 6.0f);
        S = fmaf(s, x, 1.0f);
        float c = fmaf(x, -1.0f / 3628800.0f, 1.0f / 40320.0f);
        c = fmaf(c, x, -1.0f / 720.0f);
        c = fmaf(c, x, 1.0f / 24.0f);
        c = fmaf(c, x, -0.5f);
        C = fmaf(c, x, 1.0f);
    } else if (x < 2.56f) {
        float s = -1.0f / 1307674368000.0f;
        s = fmaf(s, x, 1.0f / 6227020800.0f);
        s = fmaf(s, x, -1.0f / 39916800.0f);
        s = fmaf(s, x, 1.0f / 362880.0f);
        s = fmaf(s, x, -1.0f / 5040.0f);
        s = fmaf(s, x, 1.0f / 120.0f);
        s = fmaf(s, x, -1.0f / 6.0f);
        S = fmaf(s, x, 1.0f);
        float c = -1.0f / 87178291200.0f;
        c = fmaf(c, x, 1.0f / 479001600.0f);
        c = fmaf(c, x, -1.0f / 3628800.0f);
        c = fmaf(c, x, 1.0f / 40320.0f);
        c = fmaf(c, x, -1.0f / 720.0f);
        c = fmaf(c, x, 1.0f / 24.0f);
        c = fmaf(c, x, -0.5f);
        C = fmaf(c, x, 1.0f);
    } else {
        float sn, cs;
        sincos_mod(a, sn, cs);
        S = sn / a;
        C = cs;
    }
}

// sin(a)/a alone: the S half of sinc_cos_f (same series and ranges).
__device__ __forceinline__ float sinc_f(float a)
{
    const float x = a * a;
    if (x < 0.0256f) return fmaf(fmaf(x, 1.0f / 120.0f, -1.0f / 6.0f), x, 1.0f);
    if (x < 0.25f) {
        float s = fmaf(x, -1.0f / 5040.0f, 1.0f / 120.0f);
        s = fmaf(s, x, -1.0f / 6.0f);
        return fmaf(s, x, 1.0f);
    }
    if (x < 2.56f) {
        float s = -1.0f / 1307674368000.0f;
        s = fmaf(s, x, 1.0f / 6227020800.0f);
        s = fmaf(s, x, -1.0f / 39916800.0f);
        s = fmaf(s, x, 1.0f / 362880.0f);
        s = fmaf(s, x, -1.0f / 5040.0f);
        s = fmaf(s, x, 1.0f / 120.0f);
        s = fmaf(s, x, -1.0f / 6.0f);
        return fmaf(s, x, 1.0f);
    }
    float sn, cs;
    sincos_mod(a, sn, cs);
    return sn / a;
}

// Shared-memory position swizzle for one length-2^lg sub-array: the low k
// bits are XOR-ed with the top k bits (k = 4 for lg >= 8).  Bit-reversed reads
// (the FFT output order) then spread over the banks instead of hitting one;
// runs of consecutive positions stay conflict-free.  A bijection, applied to
// every access of the sub-array.
__device__ __forceinline__ int swz(int pos, int lg)
{
    const int k = lg >= 8 ? 4 : (lg >> 1);
    return pos ^ ((pos >> (lg - k)) & ((1 << k) - 1));
}

// 2^e as a double for -1022 <= e <= 1023, built from its bit pattern
__device__ __forceinline__ double exp2_int(int e)
{
    return __longlong_as_double((long long)(1023 + e) << 52);
}

// FP64 -> FP32 with an exact power-of-two scaling, done on the integer pipe.
// Rounds to nearest (ties away), flushes results below FP32's normal range to
// signed zero and saturates to infinity above it.  (hi:lo) << 3 holds the 23
// leading mantissa bits at [22:0] and the exponent's low 9 bits at [31:23];
// subtracting (896 - e) << 23 modulo 2^32 leaves the FP32 biased exponent
// ne = ex - 896 + e there whenever 0 < ne < 255.
__device__ __forceinline__ float d2f_scaled(double x, int e)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int ne = (int)((hi >> 20) & 0x7ffu) - 896 + e;
    unsigned mag = __funnelshift_l(lo, hi, 3) - ((unsigned)(896 - e) << 23) + ((lo >> 28) & 1u);
    mag = ((unsigned)(ne - 1) < 254u) ? mag : (ne >= 255 ? 0x7f800000u : 0u);
    return __uint_as_float((hi & 0x80000000u) | (mag & 0x7fffffffu));
}

// FP32 -> FP64 (exact) on the integer pipe: exponent rebias, mantissa shift;
// FP32 zeros and subnormals give signed zero, infinities stay infinite.
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    hi = ex == 0 ? (u & 0x80000000u) : (ex == 0xffu ? (u & 0x80000000u) | 0x7ff00000u : hi);
    const unsigned lo = ex == 0 || ex == 0xffu ? 0u : (u << 29);
    return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ double2 f2d(float2 v)
{
    return make_double2(f2d_bits(v.x), f2d_bits(v.y));
}

// ----------------------------------------------------------------------------
// third body: line-of-sight velocity (gbgpu/thirdbody.py:228-380)
// ----------------------------------------------------------------------------
__device__ double vlos_fp64(double t, const Bin &B)
{
    // Kepler inverse exactly as gbgpu/thirdbody.py:243-320
    double l = B.n2 * (t - B.T2);
    double e = B.e2;
    bool neg = l < 0.0;
    l = fabs(l);
    bool over2pi = l > 2.0 * kPi;
    double mult = 0.0;
    if (over2pi) {
        mult = floor(l / (2.0 * kPi));
        l -= mult * 2.0 * kPi;
    }
    bool overpi = l > kPi;
    if (overpi) l = 2.0 * kPi - l;
    double alpha = (1.0 - e) / (4.0 * e + 0.5);
    double beta = 0.5 * l / (4.0 * e + 0.5);
    double z = sqrt(beta * beta + alpha * alpha * alpha);
    z = neg ? beta - z : beta + z;
    z = (z < 0.0) ? -pow(-z, 1.0 / 3.0) : pow(z, 1.0 / 3.0);
    double s = z - alpha / z;
    double w = s - 0.078 * s * s * s * s * s / (1.0 + e);
    double u0 = l + e * (3.0 * w - 4.0 * w * w * w);
    double su0, cu0;
    sincos(u0, &su0, &cu0);
    double f = u0 - e * su0 - l;
    double f1 = 1.0 - e * cu0;
    double f2 = u0 - f - l;
    double f3 = 1.0 - f1;
    double f4 = -f2;
    f2 *= 0.5;
    f3 *= 0.166666666666667;
    f4 *= 0.0416666666666667;
    double u1 = -f / f1;
    double u2 = -f / (f1 + f2 * u1);
    double u3 = -f / (f1 + f2 * u2 + f3 * u2 * u2);
    double u4 = -f / (f1 + f2 * u3 + f3 * u3 * u3 + f4 * u3 * u3 * u3);
    double u = u0 + u4;
    if (overpi) u = 2.0 * kPi - u;
    if (over2pi) u = 2.0 * kPi * mult + u;
    if (neg) u = -u;
    // true anomaly (gbgpu/thirdbody.py:339-350)
    if (e > 1e-6) {
        double bt = (1.0 - sqrt(1.0 - e * e)) / e;
        double su, cu;
        sincos(u, &su, &cu);
        u += 2.0 * atan2(bt * su, 1.0 - bt * cu);
    }
    return B.A2 * (sin(u + B.varpi) + e * sin(B.varpi));
}

// Same model with the Kepler solve in FP32: eccentric anomaly u for a mean
// anomaly l in [0, pi] (Mikkola's starter and a fourth-order Newton step, as
// the FP64 form).
__device__ __forceinline__ float kepler_solve_f(float l, float e)
{
    float alpha = (1.0f - e) / (4.0f * e + 0.5f);
    float beta = 0.5f * l / (4.0f * e + 0.5f);
    float z = sqrtf(beta * beta + alpha * alpha * alpha);
    z = cbrtf(beta + z);
    float s = z - alpha / z;
    float s2 = s * s;
    float w = s - 0.078f * s2 * s2 * s / (1.0f + e);
    float u0 = l + e * (3.0f * w - 4.0f * w * w * w);
    float su0, cu0;
    sincosf(u0, &su0, &cu0);
    float f = u0 - e * su0 - l;
    float f1 = 1.0f - e * cu0;
    float f2 = 0.5f * (e * su0);
    float f3 = (1.0f / 6.0f) * (e * cu0);
    float f4 = -(1.0f / 24.0f) * (e * su0);
    float u1 = -f / f1;
    float u2 = -f / (f1 + f2 * u1);
    float u3 = -f / (f1 + f2 * u2 + f3 * u2 * u2);
    float u4 = -f / (f1 + f2 * u3 + f3 * u3 * u3 + f4 * u3 * u3 * u3);
    return u0 + u4;
}

// Eccentric anomaly (mod 2 pi) at the delayed time xi (a float pair): the
// mean anomaly M = n2 (xi - T2) and its reduction to [-pi, pi] in float-pair
// arithmetic (~1e-13 rad), then the FP32 solve on |M| with the sign put back
// (only sin/cos of the anomaly are used, so the reduction changes nothing).
// Also returns M itself (unreduced, FP32).
__device__ __forceinline__ float kepler_u_df(dfl xi, const Bin &B, float &Mout)
{
    const dfl M = df_mul(B.n2d, df_add(xi, df_neg(B.T2d)));
    Mout = M.h + M.l;
    const float q = rintf(M.h * (float)kInvTwoPi);
    const dfl r = df_add(M, df_neg(df_mul_f(df_from(kTwoPi), q)));
    const float l = r.h + r.l;
    const float u = kepler_solve_f(fminf(fabsf(l), (float)kPi), B.e2f);
    return l < 0.0f ? -u : u;
}

// v_LOS of the FP32 Kepler solve, A2 (sin(phi + varpi) + e sin varpi) with
// the true anomaly phi from u, and its time derivative
// dv/dt = A2 cos(phi + varpi)
// dphi/dM n2, with dphi/dM = sqrt(1 - e^2) / (1 - e cos u)^2 (1 / (1 - e cos u)
// below e = 1e-6, where the model takes phi = u).
__device__ float vlos_dt_mixed(dfl t, const Bin &B, float &dvdt)
{
    float M;
    const float u = kepler_u_df(t, B, M);
    const float e = B.e2f;
    float su, cu;
    sincosf(u, &su, &cu);
    const float ic = 1.0f / (1.0f - e * cu);
    float phi = u, dphi_dM = ic;
    if (e > 1e-6f) {
        const float sq = sqrtf(1.0f - e * e);
        const float bt = (1.0f - sq) / e;
        phi += 2.0f * atan2f(bt * su, 1.0f - bt * cu);
        dphi_dM = sq * ic * ic;
    }
    float sp, cp;
    sincosf(phi + B.varpif, &sp, &cp);
    dvdt = B.A2f * cp * dphi_dM * B.n2d.h;
    return B.A2f * (sp + e * B.sinvarpif);
}

// v_LOS (as vlos_dt_mixed) and its derivatives dv[0..4] = d/d(A2, varpi, e2,
// P2 [yr], T2 [yr]), dv[5] = d/dt.  With c = 1 - e cos u and M = n2 (t - T2):
// du/dM = 1/c, du/de = sin u / c (Kepler), and for the true anomaly
// dphi/du = sqrt(1-e^2)/c, dphi/de|u = sin u / (sqrt(1-e^2) c); below
// e = 1e-6 the model takes phi = u (gbgpu/thirdbody.py:339-350).
// n2 = 2 pi / (P2 yr) and T2 [s] = T2 yr give dM/dP2 = -M/P2 and
// dM/dT2 = -n2 yr = -2 pi / P2.
__device__ float vlos_grad_mixed(dfl t, const Bin &B, float cosvarpi, float P2yr, float dv[6])
{
    float M;
    const float u = kepler_u_df(t, B, M);
    const float e = B.e2f;
    float su, cu;
    sincosf(u, &su, &cu);
    const float c = 1.0f - e * cu;
    const float ic = 1.0f / c;
    float phi = u, dphi_dM, dphi_de;
    if (e > 1e-6f) {
        const float sq = sqrtf(1.0f - e * e);
        const float bt = (1.0f - sq) / e;
        phi += 2.0f * atan2f(bt * su, 1.0f - bt * cu);
        dphi_dM = sq * ic * ic;
        dphi_de = su * ic * (sq * ic + 1.0f / sq);
    } else {
        dphi_dM = ic;
        dphi_de = su * ic;
    }
    float sp, cp;
    sincosf(phi + B.varpif, &sp, &cp);
    const float A = B.A2f;
    dv[0] = sp + e * B.sinvarpif;
    dv[1] = A * fmaf(e, cosvarpi, cp);
    dv[2] = A * fmaf(cp, dphi_de, B.sinvarpif);
    const float dvdM = A * cp * dphi_dM;
    const float iP2 = 1.0f / P2yr;
    dv[3] = dvdM * M * -iP2;
    dv[4] = dvdM * (float)(-kTwoPi) * iP2;
    dv[5] = dvdM * B.n2d.h;
    return A * dv[0];
}

// ----------------------------------------------------------------------------
// per-binary set-up (gbgpu.py:212-266, 296-309)
// ----------------------------------------------------------------------------
__device__ void setup_bin(Bin &B, const KParams &K, int b, int N, int mode)
{
    const gbx_wave_args &a = K.a;
    const int nb = a.num_bin;
    const double *p = a.params;
    double amp = p[b], f0 = p[nb + b], fdot = p[2 * nb + b], fddot = p[3 * nb + b];
    double phi0 = p[4 * nb + b], iota = p[5 * nb + b], psi = p[6 * nb + b];
    double lam = p[7 * nb + b], beta = p[8 * nb + b];
    const double T = a.T;
    B.b = b;
    B.valid = 1;
    B.f0 = f0; B.fdot = fdot; B.fddot = fddot; B.phi0 = phi0;
    double q = rint(f0 * T);
    // om - 2 pi q/T cancels about seven digits; the two products are rounded
    // separately (no FMA contraction) so the phase slope carries the same
    // rounding as the reference's (om - df) (gbgpu.py:462-464, 497)
    B.om = __dmul_rn(2.0 * kPi, f0);
    B.om_m_dfa = __dsub_rn(B.om, __dmul_rn(2.0 * kPi, q / T));
    B.pifdot = kPi * fdot;
    B.pi3fddot = (1.0 / 3.0 * kPi) * fddot;
    double ci = cos(iota);
    double s2p, c2p;
    sincos(2.0 * psi, &s2p, &c2p);
    double Ap = 1.0 + ci * ci, Ac = -2.0 * ci;
    B.DP = make_double2(Ap * c2p, -Ac * s2p);
    B.DC = make_double2(-Ap * s2p, -Ac * c2p);
    double theta = kPi / 2.0 - beta;
    double st, ct, sp, cp;
    sincos(theta, &st, &ct);
    sincos(lam, &sp, &cp);
    double u[3] = {ct * cp, ct * sp, -st};
    double v[3] = {sp, -cp, 0.0};
    B.k[0] = -st * cp; B.k[1] = -st * sp; B.k[2] = -ct;
    const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
    if (a.precision == GBX_PAIR) {
        for (int c = 0; c < 3; c++) B.pr.ud[c] = df_from(u[c]);
        for (int c = 0; c < 2; c++) B.pr.vd[c] = df_from(v[c]);
        B.pr.DP = {df_from(B.DP.x), df_from(B.DP.y)};
        B.pr.DC = {df_from(B.DC.x), df_from(B.DC.y)};
    } else {
        for (int c = 0; c < 6; c++) {
            B.q.ep[c] = v[ia[c]] * v[ib[c]] - u[ia[c]] * u[ib[c]];
            B.q.ec[c] = u[ia[c]] * v[ib[c]] + v[ia[c]] * u[ib[c]];
        }
    }
    for (int c = 0; c < 3; c++) {
        B.kf[c] = (float)B.k[c];
        B.uf[c] = (float)u[c];
        B.vf[c] = (float)v[c];
        B.kd[c] = df_from(B.k[c]);
    }
    B.omd = df_from(B.om);
    B.omdfad = df_from(B.om_m_dfa);
    B.phi0d = df_from(phi0);
    B.pfd = df_from(B.pifdot);
    B.tpfd = df_from(2.0 * B.pifdot);
    B.p3d = df_from(B.pi3fddot);
    B.pfddd = df_from(kPi * fddot);
    B.DPf = make_float2((float)B.DP.x, (float)B.DP.y);
    B.DCf = make_float2((float)B.DC.x, (float)B.DC.y);
    B.f0f = (float)f0; B.fdotf = (float)fdot; B.fddotf = (float)fddot;
    {
        // f/fstar with the constant term kept as an unevaluated float pair so
        // the FP32 transfer frequency carries no per-binary rounding bias
        const double fstar = K.fstar;
        double w0 = f0 / fstar;
        B.w0h = (float)w0;
        B.w0l = (float)(w0 - (double)B.w0h);
        const double w1 = fdot / fstar;
        B.w1 = (float)w1;
        B.w1l = (float)(w1 - (double)B.w1);
        B.w2 = (float)(0.5 * fddot / fstar);
    }
    // start index, bit-exact with round(((q - N/2)/T)/(1/T))  (gbgpu.py:296, 387)
    double fmin = (q - (double)N / 2.0) / T;
    double kmin = rint(fmin / (1.0 / T));
    B.start = (int)kmin - a.start_freq_ind;
    // output scaling (gbgpu.py:298-309): amp * 0.5 T / N [* 2i sin 2wL e^{-2iwL}]
    double fc = 0.5 * T / (double)N;
    double2 sc = make_double2(amp * fc, 0.0);
    if (a.tdi2 == GBX_TDI2_BIT) {
        double omL = 2.0 * kPi * f0 * (a.armlength / kCSI);
        double s2, c2;
        sincos(2.0 * omL, &s2, &c2);
        // 2i s (c - i s) = 2 s^2 + 2i s c
        double2 t2 = make_double2(2.0 * s2 * s2, 2.0 * s2 * c2);
        sc = make_double2(fc * t2.x * amp, fc * t2.y * amp);
    }
    B.scale = sc;
    if (a.nparams >= 14) {
        B.A2 = p[9 * nb + b];
        B.varpi = p[10 * nb + b];
        B.e2 = p[11 * nb + b];
        double P2 = p[12 * nb + b];
        const double n2 = 2.0 * kPi / (P2 * a.year), T2 = p[13 * nb + b] * a.year;
        if (a.precision == GBX_FP64) {
            B.n2 = n2;
            B.T2 = T2;
        } else {
            B.n2d = df_from(n2);
            B.T2d = df_from(T2);
        }
        B.A2f = (float)B.A2;
        B.e2f = (float)B.e2;
        double vr = B.varpi - 2.0 * kPi * floor(B.varpi * kInvTwoPi);
        B.varpif = (float)vr;
        B.sinvarpif = (float)sin(B.varpi);
    }
    B.di = B.ni = B.gi = 0;
    B.eS = B.eD = 0;
    if (mode == MODE_LL || mode == MODE_SWAP) {
        int di = K.data_index ? K.data_index[b] : 0;
        int ni = K.noise_index ? K.noise_index[b] : 0;
        if (di < 0 || di >= K.num_data || ni < 0 || ni >= K.num_psd) {
            flag(a.status, GBX_FLAG_INDEX);
            B.valid = 0;
            di = ni = 0;
        }
        B.di = di; B.ni = ni;
        // power-of-two scalings so that S*2^eS and d*2^eD are O(1) in FP32
        int jm = B.start + N / 2;
        jm = jm < 0 ? 0 : (jm >= K.L ? K.L - 1 : jm);
        double Sm = K.A_psd[(size_t)ni * K.L + jm];
        int lg = (Sm > 0.0 && isfinite(Sm)) ? ilogb(Sm) : 0;
        B.eS = -lg;
        B.eD = -(lg >> 1) - 14;
    } else if (mode == MODE_FILL) {
        int gi = K.group_index[b];
        if (gi < 0 || gi >= K.num_groups) {
            flag(a.status, GBX_FLAG_INDEX);
            B.valid = 0;
            gi = 0;
        }
        B.gi = gi;
        // a zero amplitude adds nothing (the samplers zero rejected proposals)
        if (amp == 0.0) B.valid = 0;
    }
}

// ----------------------------------------------------------------------------
// Unequal arms (no counterpart in the reference, whose TDI assumes one
// armlength, gbgpu.py:167-170): arm a = 12, 23, 31 has length ell_a L at the
// sample, ell_a = |r_a| with r_a = (P_j - P_i)/L from the orbit table.  Each
// link carries its own arm: transfer argument a = (f/f*)(ell_a +- k.r_a)/2 (the
// reference's (f/f*)(1 +- k.r)/2 times ell_a with r normalised), antenna
// pattern r.e.r / ell_a^2 and amplitude ell_a; the TDI delays are the phase
// factors D_a = exp(-i omL ell_a) at the instantaneous frequency
// (quasi-static: the slow part is not re-sampled at the delayed times):
//   X = -2i omL [(1 - D_31^2)(G21 + D_12 G12) - (1 - D_12^2)(G31 + D_31 G13)]
// with Y, Z cyclic, and TDI-2 multiplies X by (1 - D_12^2 D_31^2) (Y, Z
// cyclic).  With every ell_a = 1 this is the reference's fctr2 [G21 - G31 +
// (G12 - G13) fctr] (gbgpu.py:362-372), since -2i omL (1 - D^2) = 4 omL
// sin(omL) e^{-i omL}, and its TDI-2 factor 1 - D^4 = 2i sin 2wL e^{-2iwL}
// (gbgpu.py:298-309) evaluated at f(t) instead of f0.
// ----------------------------------------------------------------------------
__device__ __forceinline__ double2 one_minus(double2 z) { return make_double2(1.0 - z.x, -z.y); }

__device__ __forceinline__ void slow_unequal_fp64(const Bin &B, double tm, double fstar,
                                               const double (&r)[3][3], const double (&kdotr)[3],
                                               const double (&fonfs)[3], const double (&kp)[3],
                                               const double2 (&A)[3], int tdi, double2 out[3])
{
    double ell[3];
#pragma unroll
    for (int a = 0; a < 3; a++) ell[a] = sqrt(r[a][0] * r[a][0] + r[a][1] * r[a][1] + r[a][2] * r[a][2]);
    double2 G[6];
    const int arm[6] = {0, 1, 2, 0, 1, 2};
    const int sc[6] = {0, 1, 2, 1, 2, 0};
    const double sg[6] = {1.0, 1.0, 1.0, -1.0, -1.0, -1.0};
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const double arg = 0.5 * fonfs[sc[q]] * (ell[arm[q]] + sg[q] * kdotr[arm[q]]);
        double sn, cs;
        sincos(arg + kp[sc[q]], &sn, &cs);
        const double amp = 0.25 * sin(arg) / arg / ell[arm[q]];
        G[q] = cmul(make_double2(amp * cs, -amp * sn), A[arm[q]]);
    }
    const double f = B.f0 + B.fdot * tm + 0.5 * B.fddot * tm * tm;
    const double omL = f / fstar;
    double2 D[3], D2[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double sn, cs;
        sincos(omL * ell[a], &sn, &cs);
        D[a] = make_double2(cs, -sn);
        D2[a] = cmul(D[a], D[a]);
    }
    double2 X = csub(cmul(one_minus(D2[2]), cadd(G[3], cmul(D[0], G[0]))),
                     cmul(one_minus(D2[0]), cadd(G[2], cmul(D[2], G[5]))));
    double2 Y = csub(cmul(one_minus(D2[0]), cadd(G[4], cmul(D[1], G[1]))),
                     cmul(one_minus(D2[1]), cadd(G[0], cmul(D[0], G[3]))));
    double2 Z = csub(cmul(one_minus(D2[1]), cadd(G[5], cmul(D[2], G[2]))),
                     cmul(one_minus(D2[2]), cadd(G[1], cmul(D[1], G[4]))));
    if (tdi & GBX_TDI2_BIT) {
        X = cmul(one_minus(cmul(D2[0], D2[2])), X);
        Y = cmul(one_minus(cmul(D2[1], D2[0])), Y);
        Z = cmul(one_minus(cmul(D2[2], D2[1])), Z);
    }
    const double2 pre = make_double2(0.0, -2.0 * omL);
    out[0] = cmul(pre, X);
    out[1] = cmul(pre, Y);
    out[2] = cmul(pre, Z);
}

// ----------------------------------------------------------------------------
// slow part at one sample (gbgpu.py:399-540 and 348-375)
// writes fctr2 * {X, Y, Z} (amplitude divided out) into out[0..2]
// ----------------------------------------------------------------------------
template <bool THIRD, bool UNEQ>
__device__ __forceinline__ void slow_fp64(const Bin &B, int n, int N, double tm, int tdi,
                                          const double *__restrict__ tab, double fstar,
                                          const double *psi, const double *vl, double2 out[3])
{
    double Pc[3][3], r[3][3];
#pragma unroll
    for (int s = 0; s < 3; s++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            Pc[s][c] = __ldg(tab + (size_t)(3 * s + c) * N + n);
            r[s][c] = __ldg(tab + (size_t)(9 + 3 * s + c) * N + n);
        }
    double kdotr[3], kP[3], xi[3], fonfs[3], kp[3];
#pragma unroll
    for (int a = 0; a < 3; a++)
        kdotr[a] = B.k[0] * r[a][0] + B.k[1] * r[a][1] + B.k[2] * r[a][2];
#pragma unroll
    for (int s = 0; s < 3; s++) {
        kP[s] = B.k[0] * Pc[s][0] + B.k[1] * Pc[s][1] + B.k[2] * Pc[s][2];
        xi[s] = tm - kP[s];
        double fi = B.f0 + B.fdot * xi[s] + 0.5 * B.fddot * xi[s] * xi[s];
        if (THIRD) fi *= 1.0 + vl[s] / kCSI;
        fonfs[s] = fi / fstar;
        double argS = B.phi0 + B.om_m_dfa * tm + B.pifdot * xi[s] * xi[s] +
                      B.pi3fddot * xi[s] * xi[s] * xi[s];
        if (THIRD) argS += psi[s];
        kp[s] = B.om * kP[s] - argS;
    }
    double2 A[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double pp = quad_form(B.q.ep, r[a][0], r[a][1], r[a][2]);
        double cc = quad_form(B.q.ec, r[a][0], r[a][1], r[a][2]);
        A[a] = make_double2(pp * B.DP.x + cc * B.DC.x, pp * B.DP.y + cc * B.DC.y);
    }
    // links (ij, sym arm, spacecraft, sign of kdotr): 12,23,31,21,32,13
    double2 G[6];
    const int arm[6] = {0, 1, 2, 0, 1, 2};
    const int sc[6] = {0, 1, 2, 1, 2, 0};
    const double sg[6] = {1.0, 1.0, 1.0, -1.0, -1.0, -1.0};
    if constexpr (UNEQ) {
        slow_unequal_fp64(B, tm, fstar, r, kdotr, fonfs, kp, A, tdi, out);
        return;
    }
#pragma unroll
    for (int q = 0; q < 6; q++) {
        double arg = 0.5 * fonfs[sc[q]] * (1.0 + sg[q] * kdotr[arm[q]]);
        double sn, cs;
        sincos(arg + kp[sc[q]], &sn, &cs);
        double amp = 0.25 * sin(arg) / arg;
        double2 e = make_double2(amp * cs, -amp * sn);
        G[q] = cmul(e, A[arm[q]]);
    }
    double f = B.f0 + B.fdot * tm + 0.5 * B.fddot * tm * tm;
    double omL = f / fstar;
    double so, co;
    sincos(omL, &so, &co);
    double2 fc = make_double2(co, -so);
    double2 fc2 = make_double2(4.0 * omL * so * co, -4.0 * omL * so * so);
    // X = G21 - G31 + (G12 - G13) fc, cyclic (gbgpu.py:370-372)
    double2 X = cadd(csub(G[3], G[2]), cmul(csub(G[0], G[5]), fc));
    double2 Y = cadd(csub(G[4], G[0]), cmul(csub(G[1], G[3]), fc));
    double2 Z = cadd(csub(G[5], G[1]), cmul(csub(G[2], G[4]), fc));
    out[0] = cmul(fc2, X);
    out[1] = cmul(fc2, Y);
    out[2] = cmul(fc2, Z);
}

// Spacecraft 1's delay k . P_1 / c at sample n as a float pair, from the
// orbit table's hi/lo rows: exact products (FMA), TwoSum accumulation.
__device__ __forceinline__ dfl kP1_pair(const Bin &B, const float *tabf, int N, int n)
{
    dfl P[3];
#pragma unroll
    for (int c = 0; c < 3; c++)
        P[c] = {__ldg(tabf + (size_t)(9 + c) * N + n), __ldg(tabf + (size_t)(18 + c) * N + n)};
    float p0 = B.kd[0].h * P[0].h, p1 = B.kd[1].h * P[1].h, p2 = B.kd[2].h * P[2].h;
    float e = fmaf(B.kd[0].h, P[0].h, -p0);
    e += fmaf(B.kd[1].h, P[1].h, -p1);
    e += fmaf(B.kd[2].h, P[2].h, -p2);
#pragma unroll
    for (int c = 0; c < 3; c++) e = fmaf(B.kd[c].h, P[c].l, fmaf(B.kd[c].l, P[c].h, e));
    const dfl s01 = df_two_sum(p0, p1);
    const dfl s012 = df_two_sum(s01.h, p2);
    return df_fast(s012.h, (s01.l + s012.l) + e);
}

// Mixed form: the carrier phase om k.P - argS (gbgpu.py:495-505), the delays
// k.P/c and the delayed times are evaluated in float-pair arithmetic (about
// 48 bits, so ~1e-12 rad at 100 rad) and reduced modulo 2 pi; everything else
// is FP32.
template <bool THIRD, bool STORE_E = false>
__device__ __forceinline__ void slow_mixed(const Bin &B, int n, int N, dfl step, float Loc,
                                           const double *__restrict__ tab,
                                           const dfl *psi, const float *vl, float2 out[3],
                                           float2 *Eout = nullptr)
{
    const float *tabf = reinterpret_cast<const float *>(tab + (size_t)18 * N);
    const dfl twopi = df_from(kTwoPi);
    const float inv2pi = (float)kInvTwoPi;
    // arm vectors r_12, r_23 from the table; r_31 = -(r_12 + r_23) closes the
    // triangle, so arm 3's projections are minus the sum of the other two
    float r[2][3];
#pragma unroll
    for (int a = 0; a < 2; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) r[a][c] = __ldg(tabf + (size_t)(3 * a + c) * N + n);
    float kdotr[3], fonfs[3], phh[3], phl[3], dlt[3], sml[3];
#pragma unroll
    for (int a = 0; a < 2; a++)
        kdotr[a] = fmaf(B.kf[0], r[a][0], fmaf(B.kf[1], r[a][1], B.kf[2] * r[a][2]));
    kdotr[2] = -(kdotr[0] + kdotr[1]);
    const dfl tm = df_mul_f(step, (float)n);                 // n T/N
    // With xi = tm - kP the carrier phase om kP - argS (gbgpu.py:495-505)
    // expands exactly into a spacecraft-independent part and powers of kP:
    //   om kP - phi0 - (om - df) tm - pi fdot xi^2 - pi/3 fddot xi^3
    //   = Phi0(tm) + kP w(tm) - pi kP^2 fd(tm) + pi/3 fddot kP^3
    // Phi0 = -phi0 - (om - df) tm - pi fdot tm^2 - pi/3 fddot tm^3,
    // w = 2 pi (f0 + fdot tm + fddot tm^2 / 2), fd = fdot + fddot tm.
    // Phi0 and w are float pairs evaluated once per sample; the kP^2 and kP^3
    // terms are below 1e-8 rad and need only FP32.
    const float tf = tm.h;
    dfl Phi0 = df_add(df_mul(B.omdfad, tm), B.phi0d);
    const dfl tm2 = df_mul(tm, tm);
    Phi0 = df_add(Phi0, df_mul(tm2, df_fast(B.pfd.h, fmaf(B.p3d.h, tf, B.pfd.l))));
    Phi0 = df_neg(Phi0);
    const dfl wt = df_add(B.omd, df_add(df_mul(B.tpfd, tm), dfl{B.pfddd.h * tf * tf, 0.0f}));
    const float fdt = fmaf(B.fddotf, tf, B.fdotf);
    const dfl kP0 = kP1_pair(B, tabf, N, n);
    // its phase, reduced mod 2 pi
    dfl ph0 = df_add(Phi0, df_mul(kP0, wt));
    if (!THIRD) {
        const float q = rintf(ph0.h * inv2pi);
        ph0 = df_add(ph0, df_neg(df_mul_f(twopi, q)));
    }
    // spacecraft 2 and 3 differ by k.(P_s - P_1)/c = (L/c) k.r (r_12 and -r_31,
    // |.| <= L/c = 8.3 s): the carrier phase moves by that times w (<= 1.3 rad
    // below 25 mHz), added in FP32 to the float pair of spacecraft 1
    const float dk[3] = {0.0f, Loc * kdotr[0], -Loc * kdotr[2]};
#pragma unroll
    for (int s = 0; s < 3; s++) {
        const float kPf = kP0.h + dk[s];
        const float small = kPf * kPf * fmaf(kPf, (1.0f / 3.0f) * B.pfddd.h, -(float)kPi * fdt);
        dfl ph = ph0;
        if (s > 0) {
            const dfl d = df_two_sum(ph0.h, dk[s] * wt.h);
            ph = dfl{d.h, d.l + ph0.l};
        }
        ph.l += small;
        if (THIRD) {
            ph = df_add(ph, df_neg(psi[s]));
            const float q = rintf(ph.h * inv2pi);
            ph = df_add(ph, df_neg(df_mul_f(twopi, q)));
        }
        phh[s] = ph.h;
        phl[s] = ph.l;
        // FP32: instantaneous frequency over the transfer frequency, and
        // f(t)/f* - f(xi)/f* = kP (w1 + w2 (t + xi)) formed directly (tiny)
        const float xf = tf - kPf;
        float fo = B.w0h + fmaf(fmaf(B.w2, xf, B.w1), xf, B.w0l);
        if (THIRD) fo *= 1.0f + vl[s] * (float)(1.0 / kCSI);
        fonfs[s] = fo;
        dlt[s] = kPf * fmaf(B.w2, tf + xf, B.w1);
        sml[s] = small;
    }
    // r.e+.r = (r.v)^2 - (r.u)^2, r.ex.r = 2 (r.u)(r.v)  (v has no z component)
    float ru[3], rv[3];
#pragma unroll
    for (int a = 0; a < 2; a++) {
        ru[a] = fmaf(B.uf[0], r[a][0], fmaf(B.uf[1], r[a][1], B.uf[2] * r[a][2]));
        rv[a] = fmaf(B.vf[0], r[a][0], B.vf[1] * r[a][1]);
    }
    ru[2] = -(ru[0] + ru[1]);
    rv[2] = -(rv[0] + rv[1]);
    float2 A[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float pp = fmaf(rv[a], rv[a], -ru[a] * ru[a]);
        const float cc = 2.0f * ru[a] * rv[a];
        A[a] = make_float2(fmaf(pp, B.DPf.x, cc * B.DCf.x), fmaf(pp, B.DPf.y, cc * B.DCf.y));
    }
    // links 12, 23, 31, 21, 32, 13: G = 1/4 sinc(a) exp(-i a) exp(-i phase_s)
    // A_arm (gbgpu.py:509-525)
    float2 G[6];
    if constexpr (THIRD) {
        // exp(-i phase_s) per spacecraft (the Doppler phases differ between
        // spacecraft), the pair's low part applied to first order
        float Er[3], Ei[3];
#pragma unroll
        for (int s = 0; s < 3; s++) {
            float sn, cs;
            sincos_mod(phh[s], sn, cs);
            Er[s] = fmaf(sn, -phl[s], cs);
            Ei[s] = -fmaf(cs, phl[s], sn);
            if (STORE_E) Eout[s] = make_float2(Er[s], Ei[s]);
        }
        const int arm[6] = {0, 1, 2, 0, 1, 2};
        const int sc[6] = {0, 1, 2, 1, 2, 0};
        const float sg[6] = {1.f, 1.f, 1.f, -1.f, -1.f, -1.f};
#pragma unroll
        for (int q = 0; q < 6; q++) {
            const int s = sc[q];
            float a = 0.5f * fonfs[s] * fmaf(sg[q], kdotr[arm[q]], 1.0f);
            float S, C;
            sinc_cos_f(a, S, C);
            const float aS = a * S;          // sin(a)
            const float t = 0.25f * S;
            // (C - i aS)(Er + i Ei)
            float2 e = make_float2(t * fmaf(C, Er[s], aS * Ei[s]), t * fmaf(C, Ei[s], -aS * Er[s]));
            G[q] = cmul(e, A[arm[q]]);
        }
    } else {
        // Each link carries its spacecraft's carrier in one exponential of the
        // summed angle a + phase_s (the angle's FP32 rounding and the phase's
        // low part applied to first order).  The two links of arm 12 -> (a+1)
        // carry angles a+ + phase_a and a- + phase_(a+1) whose difference is
        //   d = [dlt_a (1 + k.r) - dlt_(a+1) (1 - k.r)] / 2 + (kP^2 terms),
        // with dlt_s = f(t)/f* - f(xi_s)/f* (the phases differ by (L/c) k.r
        // w(t) = k.r f(t)/f*), |d| < 1e-7 rad: the second exponential is the
        // first one times (1 - i d), d formed from its small parts.
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int s2 = a == 2 ? 0 : a + 1;
            const float ap = 0.5f * fonfs[a] * (1.0f + kdotr[a]);
            const float am = 0.5f * fonfs[s2] * (1.0f - kdotr[a]);
            const dfl th = df_two_sum(phh[a], ap);
            const float thl = th.l + phl[a];
            float sn, cs;
            sincos_mod(th.h, sn, cs);
            const float2 eA = cmul(make_float2(fmaf(sn, -thl, cs), -fmaf(cs, thl, sn)), A[a]);
            const float tp = 0.25f * sinc_f(ap), tq = 0.25f * sinc_f(am);
            G[a] = make_float2(tp * eA.x, tp * eA.y);
            const float d = fmaf(0.5f * dlt[a], 1.0f + kdotr[a], -0.5f * dlt[s2] * (1.0f - kdotr[a])) +
                            (sml[s2] - sml[a]);
            G[a + 3] = make_float2(tq * fmaf(d, eA.y, eA.x), tq * fmaf(-d, eA.x, eA.y));
        }
        if (STORE_E) {
#pragma unroll
            for (int s = 0; s < 3; s++) {
                float sn, cs;
                sincos_mod(phh[s], sn, cs);
                Eout[s] = make_float2(fmaf(sn, -phl[s], cs), -fmaf(cs, phl[s], sn));
            }
        }
    }
    float omL = B.w0h + fmaf(fmaf(B.w2, tf, B.w1), tf, B.w0l);
    float so, co;
    sincos_mod(omL, so, co);
    float2 fc = make_float2(co, -so);
    float g4 = 4.0f * omL * so;
    float2 fc2 = make_float2(g4 * co, -g4 * so);
    float2 X = cadd(csub(G[3], G[2]), cmul(csub(G[0], G[5]), fc));
    float2 Y = cadd(csub(G[4], G[0]), cmul(csub(G[1], G[3]), fc));
    float2 Z = cadd(csub(G[5], G[1]), cmul(csub(G[2], G[4]), fc));
    out[0] = cmul(fc2, X);
    out[1] = cmul(fc2, Y);
    out[2] = cmul(fc2, Z);
}

// ----------------------------------------------------------------------------
// In-place decimation-in-frequency FFT over `nsub` contiguous sub-arrays of
// length N = 2^lg in shared memory; the output is in bit-reversed order.
//
// Stage `hl` (half-span h = 2^hl) maps (x_i, x_{i+h}) -> (x_i + x_{i+h},
// (x_i - x_{i+h}) W_{2h}^{i mod h}).  Stages hl >= 5 run in register passes of
// up to three stages (radix-8 groups of elements 2^q apart, q >= 5, so a warp
// touches 32 consecutive addresses: no bank conflicts); the last five stages
// (h = 16 ... 1) run inside a warp on 32 consecutive elements with shuffles.
// One __syncthreads per pass: ceil((lg - 5)/3) + 1 barriers instead of lg.
// ----------------------------------------------------------------------------
template <typename R, int RB>
__device__ __forceinline__ void fft_reg_pass(typename C2<R>::T *buf, int nsub, int lg, int hl)
{
    using V = typename C2<R>::T;
    constexpr int M = 1 << RB;
    const int q = hl - RB + 1;                 // log2 of the in-group stride
    const int groups = nsub << (lg - RB);      // N / 2^RB groups per sub-array
    for (int g = threadIdx.x; g < groups; g += kBlock) {
        const int a = g >> (lg - RB);
        const int rem = g & ((1 << (lg - RB)) - 1);
        const int blk = rem >> q;
        const int r = rem & ((1 << q) - 1);
        V *sub = buf + ((size_t)a << lg);
        const int p0 = (blk << (hl + 1)) + r;
        V x[M];
#pragma unroll
        for (int m = 0; m < M; m++) x[m] = sub[swz(p0 + (m << q), lg)];
#pragma unroll
        for (int j = 0; j < RB; j++) {
            const int dm = M >> (j + 1);             // register distance of the pair
            const int hh = hl - j;                   // log2 half-span of this stage
            const int ts = kTwN >> (hh + 1);
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (m & dm) continue;
                const int rp = r + ((m & (dm - 1)) << q);
                V u = x[m], v = x[m + dm];
                x[m] = cadd(u, v);
                x[m + dm] = cmul(csub(u, v), tw<R>(rp * ts));
            }
        }
#pragma unroll
        for (int m = 0; m < M; m++) sub[swz(p0 + (m << q), lg)] = x[m];
    }
}

template <typename R>
__device__ __forceinline__ typename C2<R>::T shfl_c(typename C2<R>::T v, int o)
{
    v.x = __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y = __shfl_xor_sync(0xffffffffu, v.y, o);
    return v;
}

template <typename R>
__device__ __forceinline__ void fft_dif(typename C2<R>::T *buf, int nsub, int lg)
{
    using V = typename C2<R>::T;
    // register passes for the stages with half-span >= 32
    int hl = lg - 1;
    while (hl >= 5) {
        const int rb = (hl - 4) >= 3 ? 3 : (hl - 4);
        if (rb == 3) fft_reg_pass<R, 3>(buf, nsub, lg, hl);
        else if (rb == 2) fft_reg_pass<R, 2>(buf, nsub, lg, hl);
        else fft_reg_pass<R, 1>(buf, nsub, lg, hl);
        hl -= rb;
        __syncthreads();
    }
    // the last five stages inside a warp: lane l holds element 32c + l.  The
    // lower lane of a pair keeps x + y, the upper one (y - x) W: both are
    // (sg x + y) w' with sg = +-1 and w' = 1 on lower lanes (and in the last
    // stage, whose twiddles are all 1), so the stage is branch-free.
    // Half-span 2 takes W^0 = 1 and W^(kTwN/4) = -i (sincospi is exact
    // there): a swap and a sign on the upper odd lanes instead of a product.
    const int lane = threadIdx.x & 31;
    V w[3];
    R sg[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const int hh = 4 - k;                       // half-span 2^hh = 16 >> k
        const bool up = (lane & (16 >> k)) != 0;
        sg[k] = up ? (R)-1 : (R)1;
        if (k < 3) {
            const int rp = lane & ((1 << hh) - 1);
            w[k] = up ? tw<R>(rp * (kTwN >> (hh + 1))) : V{(R)1, (R)0};
        }
    }
    const bool mi = (lane & 3) == 3;                // upper lane of half-span 2, W = -i
    const int chunks = (nsub << lg) >> 5;
    for (int c = threadIdx.x >> 5; c < chunks; c += kBlock >> 5) {
        const int e = (c << 5) + lane;
        const int idx = ((e >> lg) << lg) + swz(e & ((1 << lg) - 1), lg);
        V x = buf[idx];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const V y = shfl_c<R>(x, 16 >> k);
            const V d = {fma(sg[k], x.x, y.x), fma(sg[k], x.y, y.y)};
            if (k < 3) x = cmul(d, w[k]);
            else if (k == 3) x = mi ? V{d.y, -d.x} : d;
            else x = d;
        }
        buf[idx] = x;
    }
    __syncthreads();
}

// ----------------------------------------------------------------------------
// the kernel
// ----------------------------------------------------------------------------
// Third-body pre-passes (gbgpu/thirdbody.py:155-226) for a tile of cnt
// binaries with N = 2^lg samples:
//   A) v_LOS at every (sample, spacecraft) -> vl, and g = v_LOS f_GW;
//   B) trapezoid increments (xi_n - xi_{n-1}) (g_{n-1} + g_n) pi / c -> inc;
//   C) their inclusive prefix sum along n -> psi (the phase added to argS).
// FP64 throughout; inc is scratch of 3 cnt N doubles.
// Called by every thread of the block (contains barriers).
__device__ __forceinline__ void third_prepass(const Bin *bins, const double *__restrict__ tab,
                                              int cnt, int lg, double step, double *psi, double *vl,
                                              double *inc)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = 1 << lg, S = cnt << lg;
    for (int m = tid; m < S; m += kBlock) {
        const int p = m >> lg, n = m & (N - 1);
        const Bin &B = bins[p];
        const double tm = (double)n * step;
        if (!B.valid) {                       // outputs unused: no Kepler solves
#pragma unroll
            for (int s = 0; s < 3; s++) {
                psi[(p * 3 + s) * N + n] = 0.0;
                vl[(p * 3 + s) * N + n] = 0.0;
            }
            continue;
        }
#pragma unroll
        for (int s = 0; s < 3; s++) {
            double kP = B.k[0] * __ldg(tab + (size_t)(3 * s) * N + n) +
                        B.k[1] * __ldg(tab + (size_t)(3 * s + 1) * N + n) +
                        B.k[2] * __ldg(tab + (size_t)(3 * s + 2) * N + n);
            double xi = tm - kP;
            double v = vlos_fp64(xi, B);
            double fgw = B.f0 + B.fdot * xi + 0.5 * B.fddot * xi * xi;
            psi[(p * 3 + s) * N + n] = v * fgw;
            vl[(p * 3 + s) * N + n] = v;
        }
    }
    __syncthreads();
    for (int m = tid; m < S; m += kBlock) {
        const int p = m >> lg, n = m & (N - 1);
        const Bin &B = bins[p];
#pragma unroll
        for (int s = 0; s < 3; s++) {
            double v = 0.0;
            if (n > 0) {
                double d = step;
#pragma unroll
                for (int c = 0; c < 3; c++)
                    d -= B.k[c] * (__ldg(tab + (size_t)(3 * s + c) * N + n) -
                                   __ldg(tab + (size_t)(3 * s + c) * N + n - 1));
                // xi_n - xi_{n-1} = step - (kP_n - kP_{n-1})
                v = d * (psi[(p * 3 + s) * N + n - 1] + psi[(p * 3 + s) * N + n]) / 2.0 *
                    kPi * 2.0 / kCSI;
            }
            inc[(p * 3 + s) * N + n] = v;
        }
    }
    __syncthreads();
    // warp per (binary, spacecraft) row
    const int chunk = N >> 5;
    for (int row = warp; row < 3 * cnt; row += kBlock / 32) {
        const double *src = inc + (size_t)row * N + lane * chunk;
        double *dst = psi + (size_t)row * N + lane * chunk;
        double t = 0.0;
        for (int c = 0; c < chunk; c++) t += src[c];
        double incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            double y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        double run = incl - t;
        for (int c = 0; c < chunk; c++) {
            run += src[c];
            dst[c] = run;
        }
    }
    __syncthreads();
}

// Third-body pre-passes of the mixed form for a tile of cnt binaries with
// N = 2^lg samples (the same model as third_prepass above, without FP64 work
// per spacecraft):
//   A) spacecraft 1: delayed time in FP64, one Kepler solve for v_LOS and
//      dv/dt (vlos_dt_mixed); spacecraft 2, 3: v_LOS linearised in their
//      k.P/c offsets (FP32, <= L/c = 8.3 s; the second-order error is below
//      3e-9 v for P2 >= 1 yr); g = v_LOS f_GW in FP32 -> gout;
//      k.P/c of every spacecraft in FP32 -> kps (scratch);
//   B) increments (xi_n - xi_{n-1}) (g_{n-1} + g_n) pi / c with
//      xi_n - xi_{n-1} = T/N - (kP_n - kP_{n-1}) (T/N as a float pair), and
//      their inclusive prefix sum along n as float pairs -> psi.
// Called by every thread of the block (contains barriers).
__device__ __forceinline__ void third_prepass_mixed(const Bin *bins, const double *__restrict__ tab,
                                                    int cnt, int lg, dfl stp, dfl *psi,
                                                    float *vl, float *kps, float *gout)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = 1 << lg, S = cnt << lg;
    const float *tabf = reinterpret_cast<const float *>(tab + (size_t)18 * N);
    for (int m = tid; m < S; m += kBlock) {
        const int p = m >> lg, n = m & (N - 1);
        const Bin &B = bins[p];
        if (!B.valid) {                       // outputs unused: no Kepler solve
#pragma unroll
            for (int s = 0; s < 3; s++) {
                vl[(p * 3 + s) * N + n] = 0.0f;
                kps[(p * 3 + s) * N + n] = 0.0f;
                gout[(p * 3 + s) * N + n] = 0.0f;
            }
            continue;
        }
        // spacecraft 1's delayed time n T/N - k.P_1/c as a float pair
        const dfl xi0 = df_add(df_mul_f(stp, (float)n), df_neg(kP1_pair(B, tabf, N, n)));
        float dv0;
        const float v0 = vlos_dt_mixed(xi0, B, dv0);
        float kPf[3];
#pragma unroll
        for (int s = 0; s < 3; s++)
            kPf[s] = fmaf(B.kf[0], __ldg(tabf + (size_t)(9 + 3 * s) * N + n),
                          fmaf(B.kf[1], __ldg(tabf + (size_t)(9 + 3 * s + 1) * N + n),
                               B.kf[2] * __ldg(tabf + (size_t)(9 + 3 * s + 2) * N + n)));
        const float x0 = xi0.h + xi0.l;
#pragma unroll
        for (int s = 0; s < 3; s++) {
            const float dk = s ? kPf[s] - kPf[0] : 0.0f;   // xi_s = xi_1 - dk
            const float v = fmaf(-dv0, dk, v0);
            const float xf = x0 - dk;
            const float fgw = fmaf(fmaf(0.5f * B.fddotf, xf, B.fdotf), xf, B.f0f);
            vl[(p * 3 + s) * N + n] = v;
            kps[(p * 3 + s) * N + n] = kPf[s];
            gout[(p * 3 + s) * N + n] = v * fgw;
        }
    }
    __syncthreads();
    // warp per (binary, spacecraft) row; lane owns a chunk of N/32 samples
    const float k = (float)(kPi / kCSI);
    const int chunk = N >> 5;
    for (int row = warp; row < 3 * cnt; row += kBlock / 32) {
        const float *kr = kps + (size_t)row * N, *gr = gout + (size_t)row * N;
        dfl *dst = psi + (size_t)row * N;
        const int c0 = lane * chunk;
        auto inc = [&](int n) -> float {
            if (n == 0) return 0.0f;
            const float d = (stp.h - (kr[n] - kr[n - 1])) + stp.l;
            return d * (gr[n - 1] + gr[n]) * k;
        };
        dfl t = {0.0f, 0.0f};
        for (int c = 0; c < chunk; c++) t = df_add(t, dfl{inc(c0 + c), 0.0f});
        dfl incl = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const dfl y = {__shfl_up_sync(0xffffffffu, incl.h, o), __shfl_up_sync(0xffffffffu, incl.l, o)};
            if (lane >= o) incl = df_add(incl, y);
        }
        dfl run = df_add(incl, df_neg(t));
        for (int c = 0; c < chunk; c++) {
            run = df_add(run, dfl{inc(c0 + c), 0.0f});
            dst[c0 + c] = run;
        }
    }
    __syncthreads();
}

// Runs of a fill tile (MODE_FILL, called by one thread): consecutive tile
// slots with one group and ascending starts less than N apart cover one
// contiguous span of output bins.  Run r holds slots run[r] .. run[r+1]-1,
// spans lo[r] .. lo[r] + off[r+1] - off[r] - 1; an invalid binary's run is
// empty; returns the number of runs.
__device__ __forceinline__ int fill_runs(const Bin *bins, int cnt, int N, int *run, int *lo, int *off)
{
    int nr = 0, acc = 0, hi = 0;
    for (int p = 0; p < cnt; p++) {
        const Bin &B = bins[p];
        const bool join = nr > 0 && B.valid && bins[p - 1].valid && B.gi == bins[p - 1].gi &&
                          B.start >= bins[p - 1].start && B.start - bins[p - 1].start < N;
        if (!join) {
            if (nr > 0) acc += hi - lo[nr - 1];
            off[nr] = acc;
            run[nr] = p;
            lo[nr] = B.start;
            nr++;
        }
        // a run's last member ends its span; an invalid binary's run is empty
        hi = B.valid ? B.start + N : lo[nr - 1];
    }
    acc += hi - lo[nr - 1];
    off[nr] = acc;
    run[nr] = cnt;
    return nr;
}

template <typename R, int MODE, bool THIRD, bool UNEQ>
__global__ void __launch_bounds__(kBlock, sizeof(R) == 4 ? 3 : 2) wave_kernel(const KParams K)
{
    using V = typename C2<R>::T;
    // transformed channels: X, Y, Z for the waveform outputs; A, E otherwise
    constexpr int NCH = MODE == MODE_WAVE ? 3 : 2;
    const R is2 = (R)0.70710678118654752440, is6 = (R)0.40824829046386301637;
    extern __shared__ __align__(16) unsigned char smem[];
    Bin *bins = reinterpret_cast<Bin *>(smem);
    double *red = reinterpret_cast<double *>(smem + sizeof(Bin) * K.maxP);
    V *buf = reinterpret_cast<V *>(smem + sizeof(Bin) * K.maxP + sizeof(double) * red_doubles(K.maxS));
    __shared__ int s_tile;

    const gbx_wave_args &a = K.a;
    const int tid = threadIdx.x;
    const int ntiles = a.tiles ? a.ntiles : (a.num_bin + K.P - 1) / K.P;
    const double fstar = K.fstar;
    const float Loc = (float)(1.0 / (kTwoPi * fstar));         // L / c
    int iter = 0;

    for (;;) {
        if (tid == 0) {
            if (a.queue) s_tile = atomicAdd(a.queue, 1);
            else s_tile = blockIdx.x + iter * gridDim.x;
        }
        __syncthreads();
        const int tile = s_tile;
        iter++;
        if (tile >= ntiles) break;
        int lg, first, cnt;
        if (a.tiles) {
            lg = a.tiles[4 * tile];
            first = a.tiles[4 * tile + 1];
            cnt = a.tiles[4 * tile + 2];
        } else {
            lg = 31 - __clz(a.N);
            first = tile * K.P;
            cnt = min(K.P, a.num_bin - first);
        }
        const int N = 1 << lg;
        const double *tab = (lg >= 5 && lg <= GBX_MAX_LOG2N)
                                ? reinterpret_cast<const double *>(a.orbit[lg]) : nullptr;
        const int maxcnt = tile_pack(a.tile, lg, MODE == MODE_SWAP ? 2 : 1);
        if (tab == nullptr || cnt < 1 || cnt > maxcnt || first < 0 || first + cnt > a.num_bin ||
            (cnt << lg) > K.maxS || (sizeof(R) == 8 && lg > 12)) {
            flag(a.status, GBX_FLAG_TILE);
            __syncthreads();
            continue;
        }
        if (a.workspace) {
            // per-binary constants were prepared by prep_kernel: copy them in
            const int4 *src = reinterpret_cast<const int4 *>(
                static_cast<const Bin *>(a.workspace) + first);
            int4 *dst = reinterpret_cast<int4 *>(bins);
            const int n16 = cnt * (int)(sizeof(Bin) / 16);
            for (int k = tid; k < n16; k += kBlock) dst[k] = src[k];
        } else if (tid < cnt) {
            int slot = first + tid;
            int b = a.order ? a.order[slot] : slot;
            if (b < 0 || b >= a.num_bin) {
                flag(a.status, GBX_FLAG_TILE);
                memset(&bins[tid], 0, sizeof(Bin));
                bins[tid].b = -1;
            } else {
                setup_bin(bins[tid], K, b, N, MODE);
            }
        }
        __syncthreads();

        const int S = cnt << lg;                 // samples in this tile
        const double step = a.T * exp2_int(-lg);  // tm = n T/N (gbgpu.py:269), exact
        const dfl stepd = K.stepd[lg];

        double *psi = nullptr;          // FP64 form: cumulative Doppler phase
        dfl *psif = nullptr;            // mixed form: the same as float pairs
        R *vl = nullptr;
        if (THIRD) {
            if constexpr (sizeof(R) == 8) {
                psi = reinterpret_cast<double *>(buf + 3 * (size_t)maxcnt * N);
                vl = reinterpret_cast<R *>(psi + 3 * (size_t)maxcnt * N);
                third_prepass(bins, tab, cnt, lg, step, psi, reinterpret_cast<double *>(vl),
                              reinterpret_cast<double *>(buf));
            } else {
                // scratch: k.P/c and g in buf (6 floats per sample there)
                psif = reinterpret_cast<dfl *>(buf + 3 * (size_t)maxcnt * N);
                vl = reinterpret_cast<R *>(psif + 3 * (size_t)maxcnt * N);
                float *scr = reinterpret_cast<float *>(buf);
                third_prepass_mixed(bins, tab, cnt, lg, stepd, psif, reinterpret_cast<float *>(vl), scr,
                                    scr + 3 * (size_t)maxcnt * N);
            }
        }

        // slow part -> buf[(p*3 + channel)*N + n]
        for (int m = tid; m < S; m += kBlock) {
            const int p = m >> lg, n = m & (N - 1);
            const Bin &B = bins[p];
            const double tm = (double)n * step;
            double ps[3] = {0.0, 0.0, 0.0};
            dfl psf[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            R vv[3] = {0, 0, 0};
            if (THIRD) {
#pragma unroll
                for (int s = 0; s < 3; s++) {
                    if constexpr (sizeof(R) == 8) ps[s] = psi[(p * 3 + s) * N + n];
                    else psf[s] = psif[(p * 3 + s) * N + n];
                    vv[s] = vl[(p * 3 + s) * N + n];
                }
            }
            V o[3];
            if (!B.valid) {
                // nothing of this binary reaches the outputs (bad index, or a
                // zero-amplitude fill): skip the slow part
                o[0] = o[1] = o[2] = V{0, 0};
            } else if constexpr (sizeof(R) == 8) {
                double vd[3] = {(double)vv[0], (double)vv[1], (double)vv[2]};
                slow_fp64<THIRD, UNEQ>(B, n, N, tm, a.tdi2, tab, fstar, ps, vd, reinterpret_cast<double2 *>(o));
            } else {
                float vf[3] = {(float)vv[0], (float)vv[1], (float)vv[2]};
                slow_mixed<THIRD>(B, n, N, stepd, Loc, tab, psf, vf, reinterpret_cast<float2 *>(o));
            }
            if constexpr (NCH == 3) {
#pragma unroll
                for (int c = 0; c < 3; c++) buf[(p * 3 + c) * N + swz(n, lg)] = o[c];
            } else {
                // A = (Z - X)/sqrt2, E = (X - 2Y + Z)/sqrt6 (utility.py:24-38) formed
                // before the transform: the FFT is linear, so two transforms suffice
                buf[(p * 2 + 0) * N + swz(n, lg)] = {(o[2].x - o[0].x) * is2, (o[2].y - o[0].y) * is2};
                buf[(p * 2 + 1) * N + swz(n, lg)] = {(o[0].x - 2 * o[1].x + o[2].x) * is6,
                                                     (o[0].y - 2 * o[1].y + o[2].y) * is6};
            }
        }
        __syncthreads();

        fft_dif<R>(buf, NCH * cnt, lg);

        // ------------------------------------------------------------ epilogue
        if (MODE == MODE_WAVE) {
            for (int m = tid; m < S; m += kBlock) {
                const int p = m >> lg, i = m & (N - 1);
                const Bin &B = bins[p];
                if (B.b < 0) continue;
                const int pos = bitrev((i + (N >> 1)) & (N - 1), lg);   // fftshift
                V X = buf[(p * 3 + 0) * N + swz(pos, lg)], Y = buf[(p * 3 + 1) * N + swz(pos, lg)],
                  Z = buf[(p * 3 + 2) * N + swz(pos, lg)];
                const size_t o = (size_t)B.b * 3 * N + i;
                if constexpr (sizeof(R) == 8) {
                    double2 Xd = cmul(X, B.scale), Yd = cmul(Y, B.scale), Zd = cmul(Z, B.scale);
                    if (K.XYZ) {
                        K.XYZ[o] = Xd;
                        K.XYZ[o + N] = Yd;
                        K.XYZ[o + 2 * N] = Zd;
                    }
                    if (K.AET) {
                        // utility.py:24-38, with the divisions by sqrt 2, 6, 3 as
                        // products with their reciprocals (<= 1 ulp apart)
                        const double i3 = 0.57735026918962576451;
                        K.AET[o] = make_double2((Zd.x - Xd.x) * is2, (Zd.y - Xd.y) * is2);
                        K.AET[o + N] = make_double2((Xd.x - 2.0 * Yd.x + Zd.x) * is6,
                                                    (Xd.y - 2.0 * Yd.y + Zd.y) * is6);
                        K.AET[o + 2 * N] = make_double2((Xd.x + Yd.x + Zd.x) * i3,
                                                        (Xd.y + Yd.y + Zd.y) * i3);
                    }
                } else {
                    // mixed form: the channels and the scale in FP32 (the values
                    // carry FP32 accuracy), widened to FP64 on the integer pipe
                    const float2 sc = make_float2(d2f_scaled(B.scale.x, 0), d2f_scaled(B.scale.y, 0));
                    if (K.XYZ) {
                        K.XYZ[o] = f2d(cmul(X, sc));
                        K.XYZ[o + N] = f2d(cmul(Y, sc));
                        K.XYZ[o + 2 * N] = f2d(cmul(Z, sc));
                    }
                    if (K.AET) {
                        const float i3 = 0.57735026918962576451f;
                        K.AET[o] = f2d(cmul(make_float2((Z.x - X.x) * is2, (Z.y - X.y) * is2), sc));
                        K.AET[o + N] = f2d(cmul(make_float2((X.x - 2.f * Y.x + Z.x) * is6,
                                                            (X.y - 2.f * Y.y + Z.y) * is6), sc));
                        K.AET[o + 2 * N] = f2d(cmul(make_float2((X.x + Y.x + Z.x) * i3,
                                                                (X.y + Y.y + Z.y) * i3), sc));
                    }
                }
                if (i == 0 && K.start_out) K.start_out[B.b] = B.start;
            }
        } else if (MODE == MODE_SWAP) {
            // binaries 2j (current source) and 2j+1 (proposal) of the tile form a
            // pair; threads [j*Tp2, (j+1)*Tp2) walk both windows.  With r the
            // residual row and Dh = h_new - h_old:
            //   dlogL = Re<r|Dh> - 1/2 <Dh|Dh>
            //         = Re<r|h_new> - Re<r|h_old> - (<h_new|h_new> + <h_old|h_old>)/2
            //           + Re<h_old|h_new>   (cross term on the windows' overlap)
            const int Tp2 = 2 * (kBlock / maxcnt);
            const int width = Tp2 < 32 ? Tp2 : 32;
            const int pr = tid / Tp2;
            const int i0 = tid - pr * Tp2;
            typedef typename std::conditional<sizeof(R) == 8, double, float>::type Acc;
            Acc acc8[8] = {0, 0, 0, 0, 0, 0, 0, 0};   // Crn (2), Cro (2), Hn, Ho, Cx (2)
            if (2 * pr + 1 < cnt) {
                const Bin &Bo = bins[2 * pr], &Bn = bins[2 * pr + 1];
                const int po = 2 * pr, pn = 2 * pr + 1;
                if (Bo.valid && Bn.valid) {
                    bool out = false;
                    for (int e = i0; e < 2 * N; e += Tp2) {
                        const bool isnew = e < N;
                        const int i = isnew ? e : e - N;
                        const Bin &Bw = isnew ? Bn : Bo;
                        const int pw = isnew ? pn : po;
                        const int j = Bw.start + i;
                        if (j < 0 || j >= K.L) {
                            out = true;
                            continue;
                        }
                        const int pos = bitrev((i + (N >> 1)) & (N - 1), lg);
                        const V hA = buf[(pw * 2 + 0) * N + swz(pos, lg)], hE = buf[(pw * 2 + 1) * N + swz(pos, lg)];
                        const size_t jd = (size_t)Bn.di * K.L + j, jn = (size_t)Bn.ni * K.L + j;
                        const double2 dA = __ldg(K.A_data + jd), dE = __ldg(K.E_data + jd);
                        const double SA = __ldg(K.A_psd + jn), SE = __ldg(K.E_psd + jn);
                        Acc wA, wE, aR, aI, eR, eI;
                        if constexpr (sizeof(R) == 8) {
                            wA = 1.0 / SA; wE = 1.0 / SE;
                            aR = dA.x; aI = dA.y; eR = dE.x; eI = dE.y;
                        } else {
                            wA = __frcp_rn(d2f_scaled(SA, Bn.eS));
                            wE = __frcp_rn(d2f_scaled(SE, Bn.eS));
                            aR = d2f_scaled(dA.x, Bn.eD); aI = d2f_scaled(dA.y, Bn.eD);
                            eR = d2f_scaled(dE.x, Bn.eD); eI = d2f_scaled(dE.y, Bn.eD);
                        }
                        const Acc hAr = hA.x, hAi = hA.y, hEr = hE.x, hEi = hE.y;
                        // conj(r) h / S
                        const Acc cr = (aR * hAr + aI * hAi) * wA + (eR * hEr + eI * hEi) * wE;
                        const Acc ci = (aR * hAi - aI * hAr) * wA + (eR * hEi - eI * hEr) * wE;
                        const Acc hh2 = (hAr * hAr + hAi * hAi) * wA + (hEr * hEr + hEi * hEi) * wE;
                        if (isnew) {
                            acc8[0] += cr; acc8[1] += ci; acc8[4] += hh2;
                            const int k = j - Bo.start;
                            if (k >= 0 && k < N) {
                                const int pk = bitrev((k + (N >> 1)) & (N - 1), lg);
                                const V oA = buf[(po * 2 + 0) * N + swz(pk, lg)],
                                        oE = buf[(po * 2 + 1) * N + swz(pk, lg)];
                                const Acc oAr = oA.x, oAi = oA.y, oEr = oE.x, oEi = oE.y;
                                // conj(h_old) h_new / S
                                acc8[6] += (oAr * hAr + oAi * hAi) * wA + (oEr * hEr + oEi * hEi) * wE;
                                acc8[7] += (oAr * hAi - oAi * hAr) * wA + (oEr * hEi - oEi * hEr) * wE;
                            }
                        } else {
                            acc8[2] += cr; acc8[3] += ci; acc8[5] += hh2;
                        }
                    }
                    if (out) flag(a.status, GBX_FLAG_WINDOW);
                }
            }
            {
                // group trees; only the group leaders convert to FP64
                const bool leader = (tid & (width - 1)) == 0;
                const int g = tid / width;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    if constexpr (sizeof(R) == 8) {
                        double x = acc8[k];
                        for (int o = width >> 1; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                        if (leader) red[8 * g + k] = x;
                    } else {
                        dfl x = {acc8[k], 0.f};
                        for (int o = width >> 1; o > 0; o >>= 1) {
                            dfl y = {__shfl_xor_sync(0xffffffffu, x.h, o), __shfl_xor_sync(0xffffffffu, x.l, o)};
                            x = df_add(x, y);
                        }
                        if (leader) red[8 * g + k] = (double)x.h + (double)x.l;
                    }
                }
            }
            __syncthreads();
            if (2 * tid + 1 < cnt) {
                const Bin &Bo = bins[2 * tid], &Bn = bins[2 * tid + 1];
                const int per = Tp2 / width;
                double t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                for (int g = tid * per; g < (tid + 1) * per; g++)
#pragma unroll
                    for (int k = 0; k < 8; k++) t[k] += red[8 * g + k];
                double cdh = 4.0 * K.df, chh = 4.0 * K.df;
                if constexpr (sizeof(R) == 4) {
                    cdh *= exp2_int(Bn.eS - Bn.eD);
                    chh *= exp2_int(Bn.eS);
                }
                const double2 so = Bo.scale, sn = Bn.scale;
                const double rn = cmul(sn, make_double2(t[0], t[1])).x * cdh;
                const double ro = cmul(so, make_double2(t[2], t[3])).x * cdh;
                const double hn = (sn.x * sn.x + sn.y * sn.y) * t[4] * chh;
                const double ho = (so.x * so.x + so.y * so.y) * t[5] * chh;
                const double cx = cmul(make_double2(so.x, -so.y), cmul(sn, make_double2(t[6], t[7]))).x * chh;
                const bool ok = Bo.valid && Bn.valid && Bo.b >= 0 && Bn.b >= 0;
                if (Bn.b >= 0) K.dlogl[Bn.b >> 1] = ok ? (rn - ro - 0.5 * (hn + ho) + cx) : 0.0;
            }
        } else if (MODE == MODE_FILL) {
            // Pre-reduction: a run of consecutive tile slots with one group and
            // ascending starts less than N apart covers one contiguous span of
            // output bins; every bin of the span is summed over the run's
            // windows here and added with one atomic per component, instead of
            // one per window (a tile of binaries sorted by group and frequency
            // in a dense band needs a fraction of the atomics).  Unsorted
            // input gives runs of one binary: one atomic per window bin.
            __shared__ int s_run[kMaxPack + 1], s_lo[kMaxPack], s_off[kMaxPack + 1];
            __shared__ int s_nruns;
            // mixed form: the scale in FP32 (the values carry FP32 accuracy),
            // the product widened to FP64 on the integer pipe, as MODE_WAVE
            __shared__ float2 s_scf[kMaxPack];
            if (sizeof(R) == 4 && tid < cnt)
                s_scf[tid] = make_float2(d2f_scaled(bins[tid].scale.x, 0), d2f_scaled(bins[tid].scale.y, 0));
            if (tid == 0) s_nruns = fill_runs(bins, cnt, N, s_run, s_lo, s_off);
            __syncthreads();
            const int nr = s_nruns;
            const int U = s_off[nr];
            for (int m = tid; m < U; m += kBlock) {
                int r = 0;
                while (r + 1 < nr && s_off[r + 1] <= m) r++;
                const int j = s_lo[r] + (m - s_off[r]);
                if (j < 0 || j >= K.L) continue;
                double2 Ah = make_double2(0.0, 0.0), Eh = make_double2(0.0, 0.0);
                bool any = false;
                for (int p = s_run[r]; p < s_run[r + 1]; p++) {
                    const Bin &B = bins[p];
                    const int i = j - B.start;
                    if (i < 0 || i >= N) continue;
                    const int pos = bitrev((i + (N >> 1)) & (N - 1), lg);
                    const V hA = buf[(p * 2 + 0) * N + swz(pos, lg)], hE = buf[(p * 2 + 1) * N + swz(pos, lg)];
                    double2 a2, e2;
                    if constexpr (sizeof(R) == 4) {
                        a2 = f2d(cmul(hA, s_scf[p]));
                        e2 = f2d(cmul(hE, s_scf[p]));
                    } else {
                        a2 = cmul(make_double2(hA.x, hA.y), B.scale);
                        e2 = cmul(make_double2(hE.x, hE.y), B.scale);
                    }
                    // the first window adds nothing in FP64; later ones add in FP64
                    if (any) {
                        Ah = cadd(Ah, a2);
                        Eh = cadd(Eh, e2);
                    } else {
                        Ah = a2;
                        Eh = e2;
                        any = true;
                    }
                }
                const size_t o = (size_t)bins[s_run[r]].gi * K.gstride + j;
                atomicAdd(&K.A_glob[o].x, Ah.x);
                atomicAdd(&K.A_glob[o].y, Ah.y);
                atomicAdd(&K.E_glob[o].x, Eh.x);
                atomicAdd(&K.E_glob[o].y, Eh.y);
            }
        } else {  // MODE_LL
            // Threads [p*Tpb, (p+1)*Tpb) own binary p of the tile and walk its
            // window with stride Tpb, so each warp reads a contiguous run of the
            // data/PSD window.  Per-thread sums are FP64 (plain form) or FP32
            // (mixed form; N/Tpb <= 16 terms), lanes are combined with an FP64 or
            // float-pair shuffle tree, and a binary's <= 16 group partials are
            // added by one thread per (binary, term).
            const int Tpb = kBlock / maxcnt;               // 256 / binaries per tile
            const int width = Tpb < 32 ? Tpb : 32;
            const int p = tid / Tpb;
            const int i0 = tid - p * Tpb;
            typedef typename std::conditional<sizeof(R) == 8, double, float>::type Acc;
            Acc sr = 0, si = 0, sh = 0;
            // one PSD array for both channels (the usual call): the channels'
            // terms are summed, then weighted once
            const bool samepsd = K.A_psd == K.E_psd;
            if (p < cnt) {
                const Bin &B = bins[p];
                bool out = false;
                if (B.valid) {
                    for (int i = i0; i < N; i += Tpb) {
                        const int j = B.start + i;
                        if (j < 0 || j >= K.L) {
                            out = true;
                            continue;
                        }
                        const int pos = bitrev((i + (N >> 1)) & (N - 1), lg);
                        const V tA = buf[(p * 2 + 0) * N + swz(pos, lg)], tE = buf[(p * 2 + 1) * N + swz(pos, lg)];
                        const size_t jd = (size_t)B.di * K.L + j, jn = (size_t)B.ni * K.L + j;
                        const double2 dA = __ldg(K.A_data + jd), dE = __ldg(K.E_data + jd);
                        if (samepsd) {
                            const double S = __ldg(K.A_psd + jn);
                            if constexpr (sizeof(R) == 8) {
                                const double2 hA = cmul(make_double2(tA.x, tA.y), B.scale);
                                const double2 hE = cmul(make_double2(tE.x, tE.y), B.scale);
                                const double w = 1.0 / S;
                                sr += ((dA.x * hA.x + dA.y * hA.y) + (dE.x * hE.x + dE.y * hE.y)) * w;
                                si += ((dA.x * hA.y - dA.y * hA.x) + (dE.x * hE.y - dE.y * hE.x)) * w;
                                sh += ((hA.x * hA.x + hA.y * hA.y) + (hE.x * hE.x + hE.y * hE.y)) * w;
                            } else {
                                const float w = __frcp_rn(d2f_scaled(S, B.eS));
                                const float aR = d2f_scaled(dA.x, B.eD), aI = d2f_scaled(dA.y, B.eD);
                                const float eR = d2f_scaled(dE.x, B.eD), eI = d2f_scaled(dE.y, B.eD);
                                sr = fmaf(fmaf(aR, tA.x, aI * tA.y) + fmaf(eR, tE.x, eI * tE.y), w, sr);
                                si = fmaf(fmaf(aR, tA.y, -aI * tA.x) + fmaf(eR, tE.y, -eI * tE.x), w, si);
                                sh = fmaf(fmaf(tA.x, tA.x, tA.y * tA.y) + fmaf(tE.x, tE.x, tE.y * tE.y), w, sh);
                            }
                            continue;
                        }
                        const double SA = __ldg(K.A_psd + jn), SE = __ldg(K.E_psd + jn);
                        if constexpr (sizeof(R) == 8) {
                            double2 hA = cmul(make_double2(tA.x, tA.y), B.scale);
                            double2 hE = cmul(make_double2(tE.x, tE.y), B.scale);
                            const double wA = 1.0 / SA, wE = 1.0 / SE;
                            // conj(d) h / S  (gbgpu_utils.cu:172-178)
                            sr += (dA.x * hA.x + dA.y * hA.y) * wA + (dE.x * hE.x + dE.y * hE.y) * wE;
                            si += (dA.x * hA.y - dA.y * hA.x) * wA + (dE.x * hE.y - dE.y * hE.x) * wE;
                            sh += (hA.x * hA.x + hA.y * hA.y) * wA + (hE.x * hE.x + hE.y * hE.y) * wE;
                        } else {
                            const float2 hA = tA, hE = tE;
                            const float wA = __frcp_rn(d2f_scaled(SA, B.eS));
                            const float wE = __frcp_rn(d2f_scaled(SE, B.eS));
                            const float aR = d2f_scaled(dA.x, B.eD), aI = d2f_scaled(dA.y, B.eD);
                            const float eR = d2f_scaled(dE.x, B.eD), eI = d2f_scaled(dE.y, B.eD);
                            sr += fmaf(aR, hA.x, aI * hA.y) * wA + fmaf(eR, hE.x, eI * hE.y) * wE;
                            si += fmaf(aR, hA.y, -aI * hA.x) * wA + fmaf(eR, hE.y, -eI * hE.x) * wE;
                            sh += fmaf(hA.x, hA.x, hA.y * hA.y) * wA + fmaf(hE.x, hE.x, hE.y * hE.y) * wE;
                        }
                    }
                }
                if (out) flag(a.status, GBX_FLAG_WINDOW);
            }
            // lane tree within groups of `width` lanes (all lanes take part)
            double gr = 0.0, gi = 0.0, gh = 0.0;
            if constexpr (sizeof(R) == 8) {
                for (int o = width >> 1; o > 0; o >>= 1) {
                    sr += __shfl_xor_sync(0xffffffffu, sr, o);
                    si += __shfl_xor_sync(0xffffffffu, si, o);
                    sh += __shfl_xor_sync(0xffffffffu, sh, o);
                }
                gr = sr; gi = si; gh = sh;
            } else {
                dfl xr = {sr, 0.f}, xi = {si, 0.f}, xh = {sh, 0.f};
                for (int o = width >> 1; o > 0; o >>= 1) {
                    dfl yr = {__shfl_xor_sync(0xffffffffu, xr.h, o), __shfl_xor_sync(0xffffffffu, xr.l, o)};
                    dfl yi = {__shfl_xor_sync(0xffffffffu, xi.h, o), __shfl_xor_sync(0xffffffffu, xi.l, o)};
                    dfl yh = {__shfl_xor_sync(0xffffffffu, xh.h, o), __shfl_xor_sync(0xffffffffu, xh.l, o)};
                    xr = df_add(xr, yr);
                    xi = df_add(xi, yi);
                    xh = df_add(xh, yh);
                }
                // leaders keep the float pairs; the FP64 conversion happens
                // once per (binary, term) below, spread over lanes
                if ((tid & (width - 1)) == 0) {
                    float2 *red2 = reinterpret_cast<float2 *>(red);
                    const int g = tid / width;
                    red2[3 * g] = make_float2(xr.h, xr.l);
                    red2[3 * g + 1] = make_float2(xi.h, xi.l);
                    red2[3 * g + 2] = make_float2(xh.h, xh.l);
                }
            }
            if (sizeof(R) == 8 && (tid & (width - 1)) == 0) {
                const int g = tid / width;
                red[3 * g] = gr;
                red[3 * g + 1] = gi;
                red[3 * g + 2] = gh;
            }
            __syncthreads();
            // per (binary, term) sums over the binary's groups -> tsum (FP64)
            double *tsum = red + 3 * kMaxPack;
            {
                const int per = Tpb / width;
                for (int t = tid; t < 3 * cnt; t += kBlock) {
                    const int q = t / 3, c = t - 3 * q;
                    if constexpr (sizeof(R) == 8) {
                        double x = 0.0;
                        for (int g = q * per; g < (q + 1) * per; g++) x += red[3 * g + c];
                        tsum[t] = x;
                    } else {
                        const float2 *red2 = reinterpret_cast<const float2 *>(red);
                        dfl x = {0.f, 0.f};
                        for (int g = q * per; g < (q + 1) * per; g++) {
                            const float2 y = red2[3 * g + c];
                            x = df_add(x, dfl{y.x, y.y});
                        }
                        tsum[t] = (double)x.h + (double)x.l;
                    }
                }
            }
            __syncthreads();
            if (tid < cnt) {
                const Bin &B = bins[tid];
                const double tr = tsum[3 * tid], ti = tsum[3 * tid + 1], th = tsum[3 * tid + 2];
                const double s4 = 4.0 * K.df;
                double2 dh, hv;
                if constexpr (sizeof(R) == 8) {
                    dh = make_double2(s4 * tr, s4 * ti);
                    hv = make_double2(s4 * th, 0.0);
                } else {
                    // undo the power-of-two scalings and apply amp * 0.5T/N [* tdi2]
                    const double cd = s4 * exp2_int(B.eS - B.eD);
                    const double ch = s4 * exp2_int(B.eS) *
                                      (B.scale.x * B.scale.x + B.scale.y * B.scale.y);
                    dh = cmul(make_double2(cd * tr, cd * ti), B.scale);
                    hv = make_double2(ch * th, 0.0);
                }
                if (!B.valid) {
                    dh = make_double2(0.0, 0.0);
                    hv = make_double2(0.0, 0.0);
                }
                if (B.b >= 0) {
                    K.d_h[B.b] = dh;
                    K.h_h[B.b] = hv;
                }
            }
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------------------
// per-binary constants for every slot, computed once per launch by a fully
// occupied grid (one thread per binary) instead of by a few lanes of each tile
// ----------------------------------------------------------------------------
constexpr int kPrepBlock = 128;

template <int MODE>
__global__ void __launch_bounds__(kPrepBlock) prep_kernel(const KParams K)
{
    extern __shared__ __align__(16) unsigned char smem[];
    Bin *sb = reinterpret_cast<Bin *>(smem);
    const gbx_wave_args &a = K.a;
    const int s0 = blockIdx.x * kPrepBlock;
    const int slot = s0 + threadIdx.x;
    if (slot < a.num_bin) {
        int lg;
        if (a.tiles) {
            // tiles are sorted by first slot: binary search for the owning tile
            int lo = 0, hi = a.ntiles - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (a.tiles[4 * mid + 1] <= slot) lo = mid; else hi = mid - 1;
            }
            lg = a.tiles[4 * lo];
        } else {
            lg = 31 - __clz(a.N);
        }
        const int b = a.order ? a.order[slot] : slot;
        if (b < 0 || b >= a.num_bin || lg < 5 || lg > GBX_MAX_LOG2N) {
            flag(a.status, GBX_FLAG_TILE);
            memset(&sb[threadIdx.x], 0, sizeof(Bin));
            sb[threadIdx.x].b = -1;
        } else {
            setup_bin(sb[threadIdx.x], K, b, 1 << lg, MODE);
        }
    }
    __syncthreads();
    const int cnt = min(kPrepBlock, a.num_bin - s0);
    const int n16 = cnt * (int)(sizeof(Bin) / 16);
    const int4 *src = reinterpret_cast<const int4 *>(sb);
    int4 *dst = reinterpret_cast<int4 *>(static_cast<Bin *>(a.workspace) + s0);
    for (int k = threadIdx.x; k < n16; k += kPrepBlock) dst[k] = src[k];
}

constexpr int kPairMaxLog2N = 12;  // pair form: N <= 4096 (two 16-byte channels of 4096 fit)
#include "gbx_pair.cuh"
#include "gbx_grad.cuh"
#include "gbx_fisher.cuh"

// ----------------------------------------------------------------------------
// host side
// ----------------------------------------------------------------------------
// nch transformed channels per binary (3 for the waveform outputs, 2 = A, E
// otherwise); the third-body pre-passes use three slots per sample of buf as
// FP64 scratch and keep psi and v_LOS after them
static size_t smem_bytes(int prec, bool third, int maxS, int nch, int maxP)
{
    size_t head = sizeof(Bin) * (size_t)maxP + sizeof(double) * (size_t)red_doubles(maxS);
    size_t rc = prec == GBX_FP64 ? sizeof(double2) : sizeof(float2);
    size_t r = prec == GBX_FP64 ? sizeof(double) : sizeof(float);
    size_t s = head + (third ? 3 : nch) * (size_t)maxS * rc;
    if (third) s += 3 * (size_t)maxS * (sizeof(double) + r);
    return s;
}

// the pair form's layout: constants, reduction scratch, sin/cos table, buffers
static size_t pair_smem_bytes(int maxS, int nch, int maxP)
{
    return sizeof(Bin) * (size_t)maxP + sizeof(double) * (size_t)red_doubles(maxS) +
           sizeof(float4) * (size_t)kScN + (size_t)nch * maxS * sizeof(cpx);
}

// persistent launch of one tile kernel (after the per-binary prep_kernel when
// the caller gave a workspace)
template <int MODE>
static int launch_tiles(void (*kern)(const KParams), size_t sm, const KParams &K, cudaStream_t st)
{
    if (sm > 227 * 1024) return set_error(GBX_ERR_UNSUPPORTED, "tile needs %zu B of shared memory", sm);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute");
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(carveout)");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, sm);
    if (e != cudaSuccess) return cuda_error(e, "occupancy");
    if (K.a.blocks_per_sm > 0 && per_sm > K.a.blocks_per_sm) per_sm = K.a.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    int nsm = num_sms();
    int ntiles = K.a.tiles ? K.a.ntiles : (K.a.num_bin + K.P - 1) / K.P;
    int grid = per_sm * nsm;
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) return GBX_OK;
    if (K.a.queue) {
        e = cudaMemsetAsync(K.a.queue, 0, sizeof(int), st);
        if (e != cudaSuccess) return cuda_error(e, "queue reset");
    }
    if (K.a.workspace) {
        const size_t psm = sizeof(Bin) * kPrepBlock;
        auto pk = prep_kernel<MODE>;
        e = cudaFuncSetAttribute(pk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm);
        if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(prep)");
        pk<<<(K.a.num_bin + kPrepBlock - 1) / kPrepBlock, kPrepBlock, psm, st>>>(K);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_error(e, "prep_kernel launch");
    }
    kern<<<grid, kBlock, sm, st>>>(K);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "wave_kernel launch");
    return GBX_OK;
}

template <typename R, int MODE, bool THIRD, bool UNEQ = false>
static int launch_one(const KParams &K, int maxS, cudaStream_t st)
{
    const size_t sm = smem_bytes(sizeof(R) == 8 ? GBX_FP64 : GBX_MIXED, THIRD, maxS,
                                 MODE == MODE_WAVE ? 3 : 2, K.maxP);
    return launch_tiles<MODE>(wave_kernel<R, MODE, THIRD, UNEQ>, sm, K, st);
}

// most binaries in one tile of this launch (the shared memory holds their constants)
static int max_pack(const gbx_wave_args *a, int minp)
{
    if (a->tiles == nullptr) return tile_pack(a->tile, 31 - __builtin_clz((unsigned)a->N), minp);
    int mp = 1;
    for (int k = 5; k <= GBX_MAX_LOG2N; k++)
        if (a->orbit[k]) mp = max(mp, tile_pack(a->tile, k, minp));
    return mp;
}

template <int MODE>
static int dispatch(KParams &K, int maxS, cudaStream_t st)
{
    K.maxS = maxS;
    K.maxP = max_pack(&K.a, MODE == MODE_SWAP ? 2 : 1);
    const bool third = K.a.nparams >= 14;
    // unequal arms are a separate instantiation: the equal-arm kernels carry none of it
    const bool uneq = (K.a.tdi2 & GBX_TDI_UNEQUAL) != 0;
    if (uneq && third) return set_error(GBX_ERR_UNSUPPORTED, "unequal arms cover the 9-parameter model");
    if (K.a.precision == GBX_PAIR) {
        if constexpr (MODE == MODE_WAVE || MODE == MODE_LL || MODE == MODE_FILL || MODE == MODE_SWAP) {
            if (third) return set_error(GBX_ERR_UNSUPPORTED, "the pair form covers the 9-parameter model");
            return launch_tiles<MODE>(uneq ? pair_kernel<MODE, true> : pair_kernel<MODE, false>,
                                      pair_smem_bytes(maxS, MODE == MODE_WAVE ? 3 : 2, K.maxP), K, st);
        } else {
            return set_error(GBX_ERR_UNSUPPORTED, "the pair form covers the waveform, likelihood, fill and swap entry points");
        }
    }
    if (K.a.precision == GBX_FP64) {
        if (uneq) return launch_one<double, MODE, false, true>(K, maxS, st);
        return third ? launch_one<double, MODE, true>(K, maxS, st)
                     : launch_one<double, MODE, false>(K, maxS, st);
    }
    return third ? launch_one<float, MODE, true>(K, maxS, st)
                 : launch_one<float, MODE, false>(K, maxS, st);
}

// validates the shared arguments; returns max samples per tile in *maxS
static int check_wave(const gbx_wave_args *a, int *maxS)
{
    if (!a || !a->params) return set_error(GBX_ERR_ARG, "NULL wave args / params");
    if (a->num_bin < 0) return set_error(GBX_ERR_ARG, "num_bin < 0");
    if (a->nparams != 9 && a->nparams != 14) return set_error(GBX_ERR_ARG, "nparams must be 9 or 14");
    if (a->precision != GBX_FP64 && a->precision != GBX_MIXED && a->precision != GBX_PAIR)
        return set_error(GBX_ERR_ARG, "unknown precision %d", a->precision);
    if (!(a->T > 0.0) || !(a->armlength > 0.0)) return set_error(GBX_ERR_ARG, "T and armlength must be > 0");
    if (a->nparams == 14 && !(a->year > 0.0)) return set_error(GBX_ERR_ARG, "year must be > 0");
    if (a->tdi2 < 0 || a->tdi2 > (GBX_TDI2_BIT | GBX_TDI_UNEQUAL))
        return set_error(GBX_ERR_ARG, "tdi2=%d: bits GBX_TDI2_BIT and GBX_TDI_UNEQUAL only", a->tdi2);
    if ((a->tdi2 & GBX_TDI_UNEQUAL) && a->precision == GBX_MIXED)
        return set_error(GBX_ERR_UNSUPPORTED, "unequal arms are computed in the FP64 and pair forms only");
    if (a->workspace) {
        if (((uintptr_t)a->workspace & 15) != 0) return set_error(GBX_ERR_ARG, "workspace must be 16-byte aligned");
        if (a->workspace_bytes < gbx_wave_workspace_bytes(a->num_bin))
            return set_error(GBX_ERR_ARG, "workspace smaller than gbx_wave_workspace_bytes(num_bin)");
    }
    if (a->tile != 0 && (a->tile < 64 || a->tile > 4096 || (a->tile & (a->tile - 1)) != 0))
        return set_error(GBX_ERR_ARG, "tile=%d: need 0 or a power of two in [64, 4096]", a->tile);
    if (a->blocks_per_sm < 0) return set_error(GBX_ERR_ARG, "blocks_per_sm < 0");
    const int maxlg = a->precision == GBX_MIXED ? GBX_MAX_LOG2N : 12;
    if (a->tiles == nullptr) {
        int N = a->N;
        if (N < 32 || (N & (N - 1)) != 0) return set_error(GBX_ERR_UNSUPPORTED, "N=%d: need a power of two >= 32", N);
        int lg = 31 - __builtin_clz((unsigned)N);
        if (lg > maxlg) return set_error(GBX_ERR_UNSUPPORTED, "N=%d above the limit of this precision", N);
        if (!a->orbit[lg]) return set_error(GBX_ERR_ARG, "no orbit table for N=%d", N);
        *maxS = tile_pack(a->tile, lg, 1) * N;
    } else {
        if (a->ntiles < 0) return set_error(GBX_ERR_ARG, "ntiles < 0");
        // the N with a table bound the tile size
        int mx = 0;
        for (int k = 5; k <= maxlg; k++)
            if (a->orbit[k]) mx = max(mx, tile_pack(a->tile, k, 1) << k);
        if (mx == 0) return set_error(GBX_ERR_ARG, "no orbit tables");
        *maxS = mx;
    }
    return GBX_OK;
}

static KParams base_params(const gbx_wave_args *a)
{
    KParams K;
    memset(&K, 0, sizeof(K));
    K.a = *a;
    K.fstar = kCSI / (a->armlength * 2.0 * kPi);
    for (int k = 0; k <= GBX_MAX_LOG2N; k++) K.stepd[k] = df_from(ldexp(a->T, -k));
    K.Locd = df_from(a->armlength / kCSI);
    K.P = a->tiles == nullptr ? tile_pack(a->tile, 31 - __builtin_clz((unsigned)a->N), 1) : 1;
    return K;
}

}  // namespace gbx

using namespace gbx;

extern "C" size_t gbx_wave_workspace_bytes(int num_bin)
{
    if (num_bin <= 0) return 0;
    return ((size_t)num_bin * sizeof(Bin) + 255) & ~(size_t)255;
}

int gbx_twiddle_init(cudaStream_t st)
{
    tw_init_kernel<<<(kTwN / 2 + 255) / 256, 256, 0, st>>>();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "twiddle init");
    return GBX_OK;
}

extern "C" int gbx_waveform(const gbx_wave_args *a, void *XYZ_out, void *AET_out, int *start_out,
                            void *stream)
{
    int maxS = 0;
    int rc = check_wave(a, &maxS);
    if (rc) return rc;
    if (a->tiles) return set_error(GBX_ERR_ARG, "gbx_waveform takes a uniform N");
    rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    KParams K = base_params(a);
    K.XYZ = (double2 *)XYZ_out;
    K.AET = (double2 *)AET_out;
    K.start_out = start_out;
    return dispatch<MODE_WAVE>(K, maxS, (cudaStream_t)stream);
}

extern "C" int gbx_waveform_ll(const gbx_wave_args *a, const gbx_ll_args *l, void *d_h, void *h_h,
                               void *stream)
{
    int maxS = 0;
    int rc = check_wave(a, &maxS);
    if (rc) return rc;
    if (!l || !l->A_data || !l->E_data || !l->A_psd || !l->E_psd || !d_h || !h_h)
        return set_error(GBX_ERR_ARG, "NULL likelihood pointer");
    if (l->data_length <= 0 || l->num_data < 1 || l->num_psd < 1)
        return set_error(GBX_ERR_ARG, "data_length / num_data / num_psd must be positive");
    rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    KParams K = base_params(a);
    K.A_data = (const double2 *)l->A_data;
    K.E_data = (const double2 *)l->E_data;
    K.A_psd = l->A_psd;
    K.E_psd = l->E_psd;
    K.L = l->data_length;
    K.num_data = l->num_data;
    K.num_psd = l->num_psd;
    K.data_index = l->data_index;
    K.noise_index = l->noise_index;
    K.df = l->df;
    K.d_h = (double2 *)d_h;
    K.h_h = (double2 *)h_h;
    return dispatch<MODE_LL>(K, maxS, (cudaStream_t)stream);
}

extern "C" int gbx_waveform_fill(const gbx_wave_args *a, void *A_glob, void *E_glob,
                                 const int *group_index, int num_groups, int data_length,
                                 long long group_stride, void *stream)
{
    int maxS = 0;
    int rc = check_wave(a, &maxS);
    if (rc) return rc;
    if (!A_glob || !E_glob || !group_index) return set_error(GBX_ERR_ARG, "NULL fill pointer");
    if (data_length <= 0 || num_groups < 1) return set_error(GBX_ERR_ARG, "bad template shape");
    if (group_stride == 0) group_stride = data_length;
    if (group_stride < data_length) return set_error(GBX_ERR_ARG, "group_stride < data_length");
    rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    KParams K = base_params(a);
    K.A_glob = (double2 *)A_glob;
    K.E_glob = (double2 *)E_glob;
    K.group_index = group_index;
    K.num_groups = num_groups;
    K.gstride = group_stride;
    K.L = data_length;
    return dispatch<MODE_FILL>(K, maxS, (cudaStream_t)stream);
}

extern "C" int gbx_swap_ll(const gbx_wave_args *a, const gbx_ll_args *l, double *dlogl,
                           void *stream)
{
    int maxS = 0;
    int rc = check_wave(a, &maxS);
    if (rc) return rc;
    if (a->tiles || a->order) return set_error(GBX_ERR_ARG, "gbx_swap_ll takes a uniform N and no order");
    if (a->num_bin % 2) return set_error(GBX_ERR_ARG, "num_bin must be even: (old, new) pairs");
    if (!l || !l->A_data || !l->E_data || !l->A_psd || !l->E_psd || !dlogl)
        return set_error(GBX_ERR_ARG, "NULL likelihood pointer");
    if (l->data_length <= 0 || l->num_data < 1 || l->num_psd < 1)
        return set_error(GBX_ERR_ARG, "data_length / num_data / num_psd must be positive");
    rc = ensure_init((cudaStream_t)stream);
    if (rc) return rc;
    KParams K = base_params(a);
    K.P = tile_pack(a->tile, 31 - __builtin_clz((unsigned)a->N), 2);
    maxS = K.P * a->N;
    K.A_data = (const double2 *)l->A_data;
    K.E_data = (const double2 *)l->E_data;
    K.A_psd = l->A_psd;
    K.E_psd = l->E_psd;
    K.L = l->data_length;
    K.num_data = l->num_data;
    K.num_psd = l->num_psd;
    K.data_index = l->data_index;
    K.noise_index = l->noise_index;
    K.df = l->df;
    K.dlogl = dlogl;
    return dispatch<MODE_SWAP>(K, maxS, (cudaStream_t)stream);
}

extern "C" size_t gbx_grad_workspace_bytes(int num_bin)
{
    if (num_bin <= 0) return 0;
    return ((size_t)num_bin * (sizeof(Bin) + sizeof(GradExtra)) + 255) & ~(size_t)255;
}

// validates the gradient entry points' arguments (b: a copy of the caller's,
// workspace checked here, not by check_wave); *maxS as check_wave
static int check_grad(gbx_wave_args &b, const gbx_ll_args *l, int *maxS)
{
    const void *ws = b.workspace;
    const size_t wsb = b.workspace_bytes;
    b.workspace = nullptr;
    int rc = check_wave(&b, maxS);
    if (rc) return rc;
    if (b.precision != GBX_MIXED) return set_error(GBX_ERR_UNSUPPORTED, "gradients are computed in the mixed form only");
    if (b.nparams != 9 && b.nparams != 14)
        return set_error(GBX_ERR_UNSUPPORTED, "gradients cover the 9-parameter model and the 14-parameter third-body model");
    if (!ws || ((uintptr_t)ws & 15) != 0 || wsb < gbx_grad_workspace_bytes(b.num_bin))
        return set_error(GBX_ERR_ARG, "gradients need a 16-byte aligned workspace of gbx_grad_workspace_bytes(num_bin)");
    if (!l || !l->A_data || !l->E_data || !l->A_psd || !l->E_psd)
        return set_error(GBX_ERR_ARG, "NULL likelihood pointer");
    if (l->data_length <= 0 || l->num_data < 1 || l->num_psd < 1)
        return set_error(GBX_ERR_ARG, "data_length / num_data / num_psd must be positive");
    b.workspace = const_cast<void *>(ws);
    b.workspace_bytes = wsb;
    return GBX_OK;
}

static void set_ll(KParams &K, const gbx_ll_args *l)
{
    K.A_data = (const double2 *)l->A_data;
    K.E_data = (const double2 *)l->E_data;
    K.A_psd = l->A_psd;
    K.E_psd = l->E_psd;
    K.L = l->data_length;
    K.num_data = l->num_data;
    K.num_psd = l->num_psd;
    K.data_index = l->data_index;
    K.noise_index = l->noise_index;
    K.df = l->df;
}

// prep_grad_kernel + grad_kernel<third, SWAP> over the validated arguments
template <bool SWAP>
static int launch_grad(const gbx_wave_args &b, const gbx_ll_args *l, void *d_h, void *h_h,
                       double *grad, int maxS, cudaStream_t st)
{
    GradParams G;
    memset(&G, 0, sizeof(G));
    G.K = base_params(&b);
    KParams &K = G.K;
    set_ll(K, l);
    K.d_h = (double2 *)d_h;
    K.h_h = (double2 *)h_h;
    if (SWAP) {
        K.P = tile_pack(b.tile, 31 - __builtin_clz((unsigned)b.N), 2);
        maxS = K.P * b.N;
    }
    K.maxS = maxS;
    K.maxP = max_pack(&K.a, SWAP ? 2 : 1);
    G.grad = grad;
    const bool third = b.nparams == 14;
    auto kern = third ? grad_kernel<true, SWAP> : grad_kernel<false, SWAP>;
    const size_t sm = grad_smem_bytes(third, maxS, K.maxP);
    if (sm > 227 * 1024) return set_error(GBX_ERR_UNSUPPORTED, "tile needs %zu B of shared memory", sm);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(grad)");
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(grad carveout)");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, sm);
    if (e != cudaSuccess) return cuda_error(e, "occupancy(grad)");
    if (b.blocks_per_sm > 0 && per_sm > b.blocks_per_sm) per_sm = b.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    const int ntiles = b.tiles ? b.ntiles : (b.num_bin + K.P - 1) / K.P;
    int grid = per_sm * num_sms();
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) return GBX_OK;
    if (b.queue) {
        e = cudaMemsetAsync(b.queue, 0, sizeof(int), st);
        if (e != cudaSuccess) return cuda_error(e, "queue reset");
    }
    const size_t psm = (sizeof(Bin) + sizeof(GradExtra)) * kPrepBlock;
    e = cudaFuncSetAttribute(prep_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(prep_grad)");
    prep_grad_kernel<<<(b.num_bin + kPrepBlock - 1) / kPrepBlock, kPrepBlock, psm, st>>>(K);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "prep_grad_kernel launch");
    kern<<<grid, kBlock, sm, st>>>(G);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "grad_kernel launch");
    return GBX_OK;
}

extern "C" int gbx_waveform_ll_grad(const gbx_wave_args *a, const gbx_ll_args *l, void *d_h,
                                    void *h_h, double *grad, void *stream)
{
    if (!a) return set_error(GBX_ERR_ARG, "NULL wave args");
    int maxS = 0;
    gbx_wave_args b = *a;
    int rc = check_grad(b, l, &maxS);
    if (rc) return rc;
    if (!d_h || !h_h || !grad) return set_error(GBX_ERR_ARG, "NULL likelihood / gradient pointer");
    if (b.num_bin == 0) return GBX_OK;
    cudaStream_t st = (cudaStream_t)stream;
    rc = ensure_init(st);
    if (rc) return rc;
    return launch_grad<false>(b, l, d_h, h_h, grad, maxS, st);
}

extern "C" int gbx_swap_ll_grad(const gbx_wave_args *a, const gbx_ll_args *l, double *dlogl,
                                double *grad, void *stream)
{
    if (!a) return set_error(GBX_ERR_ARG, "NULL wave args");
    int maxS = 0;
    gbx_wave_args b = *a;
    int rc = check_grad(b, l, &maxS);
    if (rc) return rc;
    if (b.tiles || b.order) return set_error(GBX_ERR_ARG, "gbx_swap_ll_grad takes a uniform N and no order");
    if (b.num_bin % 2) return set_error(GBX_ERR_ARG, "num_bin must be even: (old, new) pairs");
    if (!grad) return set_error(GBX_ERR_ARG, "NULL gradient pointer");
    if (b.num_bin == 0) return GBX_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (dlogl) {
        // the change of log-likelihood itself: the swap kernel, as gbx_swap_ll
        rc = gbx_swap_ll(&b, l, dlogl, stream);
        if (rc) return rc;
    } else {
        rc = ensure_init(st);
        if (rc) return rc;
    }
    return launch_grad<true>(b, l, nullptr, nullptr, grad, maxS, st);
}

extern "C" int gbx_fisher(const gbx_wave_args *a, const double *A_psd, const double *E_psd,
                          int psd_length, int num_psd, const int *noise_index, double df,
                          double *fisher, void *stream)
{
    if (!a) return set_error(GBX_ERR_ARG, "NULL wave args");
    int maxS = 0;
    gbx_wave_args b = *a;
    gbx_ll_args l;
    memset(&l, 0, sizeof(l));
    // the likelihood arguments' checks, with the PSD rows standing in for the
    // data (never read)
    l.A_data = A_psd;
    l.E_data = E_psd;
    l.A_psd = A_psd;
    l.E_psd = E_psd;
    l.data_length = psd_length;
    l.num_data = 1;
    l.num_psd = num_psd;
    l.noise_index = noise_index;
    l.df = df;
    int rc = check_grad(b, &l, &maxS);
    if (rc) return rc;
    if (b.nparams != 9) return set_error(GBX_ERR_UNSUPPORTED, "Fisher matrices cover the 9-parameter model");
    if (b.tdi2 & GBX_TDI_UNEQUAL) return set_error(GBX_ERR_UNSUPPORTED, "Fisher matrices take equal arms");
    if (!fisher) return set_error(GBX_ERR_ARG, "NULL Fisher output");
    if (b.num_bin == 0) return GBX_OK;
    cudaStream_t st = (cudaStream_t)stream;
    rc = ensure_init(st);
    if (rc) return rc;
    FisherParams F;
    memset(&F, 0, sizeof(F));
    F.K = base_params(&b);
    KParams &K = F.K;
    set_ll(K, &l);
    K.A_data = nullptr;
    K.E_data = nullptr;
    K.data_index = nullptr;
    K.maxS = maxS;
    K.maxP = max_pack(&K.a, 1);
    F.fisher = fisher;
    const size_t sm = fisher_smem_bytes(maxS, K.maxP);
    if (sm > 227 * 1024) return set_error(GBX_ERR_UNSUPPORTED, "tile needs %zu B of shared memory (use a smaller tile)", sm);
    cudaError_t e = cudaFuncSetAttribute(fisher_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(fisher)");
    e = cudaFuncSetAttribute(fisher_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(fisher carveout)");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fisher_kernel, kBlock, sm);
    if (e != cudaSuccess) return cuda_error(e, "occupancy(fisher)");
    if (b.blocks_per_sm > 0 && per_sm > b.blocks_per_sm) per_sm = b.blocks_per_sm;
    if (per_sm < 1) per_sm = 1;
    const int ntiles = b.tiles ? b.ntiles : (b.num_bin + K.P - 1) / K.P;
    int grid = per_sm * num_sms();
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) return GBX_OK;
    if (b.queue) {
        e = cudaMemsetAsync(b.queue, 0, sizeof(int), st);
        if (e != cudaSuccess) return cuda_error(e, "queue reset");
    }
    const size_t psm = (sizeof(Bin) + sizeof(GradExtra)) * kPrepBlock;
    e = cudaFuncSetAttribute(prep_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm);
    if (e != cudaSuccess) return cuda_error(e, "cudaFuncSetAttribute(prep_grad)");
    prep_grad_kernel<<<(b.num_bin + kPrepBlock - 1) / kPrepBlock, kPrepBlock, psm, st>>>(K);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "prep_grad_kernel launch");
    fisher_kernel<<<grid, kBlock, sm, st>>>(F);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "fisher_kernel launch");
    return GBX_OK;
}

// ----------------------------------------------------------------------------
// Diagnostic entry point for the FP32 math helpers
// ----------------------------------------------------------------------------
namespace gbx {
__global__ void math_selftest_kernel(const void *x, float *out, int n, int which, int e)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (which == 2) {
        out[i] = d2f_scaled(static_cast<const double *>(x)[i], e);
        return;
    }
    const float xi = static_cast<const float *>(x)[i];
    float a, b;
    if (which == 0) sincos_mod(xi, a, b);
    else sinc_cos_f(xi, a, b);
    out[2 * i] = a;
    out[2 * i + 1] = b;
}
}  // namespace gbx

extern "C" int gbx_math_selftest(const void *x, float *out, int n, int which, int e, void *stream)
{
    if (n < 0 || (n > 0 && (!x || !out)) || which < 0 || which > 2)
        return set_error(GBX_ERR_ARG, "math selftest: bad arguments");
    if (n == 0) return GBX_OK;
    gbx::math_selftest_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(x, out, n, which, e);
    const cudaError_t err = cudaGetLastError();
    return err == cudaSuccess ? GBX_OK : cuda_error(err, "math_selftest_kernel launch");
}

// ----------------------------------------------------------------------------
// Allocation-free variant of gbx_waveform_ll.
//
// Some callers cannot allocate device memory at all: a plug-in inside a host
// application that owns every device allocation and only lends it pointers,
// or an FFI caller that binds this C ABI but has no CUDA allocator of its own.
// They cannot provide the per-binary workspace or the work-queue counter, so
// this entry point keeps both in the file-scope array below.  Every GPU that
// loads the library holds the array (4 MiB + 256 B) until the process exits.
// ----------------------------------------------------------------------------
namespace gbx {
constexpr int kNoAllocMaxBin = GBX_NOALLOC_MAX_BINS;
// 512 bytes per binary: the published size (4 MiB + 256 B) stays fixed while Bin fits
static_assert(sizeof(Bin) <= 512, "the allocation-free scratch holds 512 bytes per binary");
constexpr size_t kNoAllocWsBytes = (size_t)kNoAllocMaxBin * 512;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocWsBytes + 256];

static std::mutex g_noalloc_lock;
static void *g_noalloc_ptr[64] = {};

// The host-side name g_noalloc_scratch is only a stand-in for the device
// array; its device address comes from cudaGetSymbolAddress, once per device,
// with that device current.
static int noalloc_scratch(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(GBX_ERR_ARG, "device %d out of range", dev);
    std::lock_guard<std::mutex> g(g_noalloc_lock);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(scratch)");
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
    return GBX_OK;
}
}  // namespace gbx

extern "C" int gbx_waveform_ll_noalloc(const gbx_wave_args *a, const gbx_ll_args *l, void *d_h,
                                       void *h_h, void *stream)
{
    if (!a) return set_error(GBX_ERR_ARG, "NULL wave args");
    if (a->num_bin > kNoAllocMaxBin)
        return set_error(GBX_ERR_ARG, "num_bin %d exceeds the %d binaries of the static scratch",
                         a->num_bin, kNoAllocMaxBin);
    void *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    gbx_wave_args b = *a;
    b.workspace = scratch;
    b.workspace_bytes = kNoAllocWsBytes;
    // the queue counter lives after the workspace; it is reset on the stream
    // before every launch that uses it
    b.queue = b.tiles ? reinterpret_cast<int *>(static_cast<unsigned char *>(scratch) + kNoAllocWsBytes)
                      : nullptr;
    return gbx_waveform_ll(&b, l, d_h, h_h, stream);
}
