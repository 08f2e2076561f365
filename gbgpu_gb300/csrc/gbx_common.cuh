// Shared device helpers for the GB300 FastGB kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbgpu_gb300.h"

namespace gbx {

constexpr int kBlock = 256;        // threads per CTA for the waveform family
constexpr int kTileMin = 512;      // default samples per tile (P = kTileMin / N binaries)
constexpr int kMaxPack = 16;       // most binaries in one tile (also the most lane groups)

// binaries of N = 2^lg packed in one tile of `tile` samples (tile 0 = kTileMin)
__host__ __device__ __forceinline__ int tile_pack(int tile, int lg, int minp)
{
    int p = (tile ? tile : kTileMin) >> lg;
    p = p < minp ? minp : p;
    return p > kMaxPack ? kMaxPack : p;
}
constexpr int kTwN = 8192;         // twiddle table period (largest supported N)
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTwoPi = 6.283185307179586476925286766559005768;
constexpr double kInvTwoPi = 0.159154943091895335768883763372514362;
constexpr double kCSI = 299792458.0;

// ---------------------------------------------------------------- complex
template <typename R> struct C2;
template <> struct C2<float> { using T = float2; };
template <> struct C2<double> { using T = double2; };

__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }

template <typename V> __device__ __forceinline__ V cadd(V a, V b) { V r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { V r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename V> __device__ __forceinline__ V cmul(V a, V b)
{
    V r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// bit reversal of the low `bits` bits
__device__ __forceinline__ int bitrev(int k, int bits) { return (int)(__brev((unsigned)k) >> (32 - bits)); }

// ---------------------------------------------------------------- double-float
// Unevaluated pairs hi + lo of FP32 numbers (Dekker 1971; Knuth TAOCP vol. 2,
// 4.2.2): TwoSum and TwoProd (via FMA) are error-free, so sums and products
// of pairs carry about 48 significant bits using FP32 instructions only.
struct dfl {
    float h, l;
};
__device__ __forceinline__ dfl df_two_sum(float a, float b)
{
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ dfl df_fast(float a, float b)   // requires |a| >= |b| or a == 0
{
    float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b)
{
    dfl s = df_two_sum(a.h, b.h);
    return df_fast(s.h, s.l + (a.l + b.l));
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_fast(p, e);
}
__device__ __forceinline__ dfl df_mul_f(dfl a, float b)
{
    float p = a.h * b;
    float e = fmaf(a.h, b, -p);
    e = fmaf(a.l, b, e);
    return df_fast(p, e);
}
__host__ __device__ __forceinline__ dfl df_from(double x)
{
    float h = (float)x;
    return {h, (float)(x - (double)h)};
}
// the pair of a double known at compile time (folded by the compiler)
__host__ __device__ constexpr dfl dconst(double x)
{
    return dfl{(float)x, (float)(x - (double)(float)x)};
}

// complex number with float-pair parts (16 bytes, one vector access)
struct __align__(16) cpx {
    dfl x, y;
};

// FP64 x * 2^e as an unevaluated float pair hi + lo, built mostly on the
// integer pipe: hi carries the 24 leading significant bits, lo the next 23
// (both truncated), so |x 2^e - (hi + lo)| < 2^-46 |x 2^e|.  (hi:lo) << 3
// holds the 23 leading mantissa bits at [22:0] and the exponent's low 9 bits
// at [31:23]; subtracting (896 - e) << 23 leaves the FP32 biased exponent
// there when it is in range.  Scaled values below FP32's normal range become
// signed zero, values above it (and infinities, NaN) infinity; lo is the
// next 23 bits as an exact FP32 integer times hi's power of two times 2^-46
// (so it underflows to zero for |hi| < 2^-80).
__device__ __forceinline__ dfl d2ff_scaled(double x, int e)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int ne = (int)((hi >> 20) & 0x7ffu) - 896 + e;          // FP32 biased exponent
    unsigned mag = __funnelshift_l(lo, hi, 3) - ((unsigned)(896 - e) << 23);
    mag = ((unsigned)(ne - 1) < 254u) ? mag : (ne >= 255 ? 0x7f800000u : 0u);
    const unsigned hb = (hi & 0x80000000u) | (mag & 0x7fffffffu);
    const float r = __uint_as_float(0x4b000000u | ((lo >> 6) & 0x7fffffu)) - 8388608.0f;
    const float l = r * (__uint_as_float(hb & 0xff800000u) * 0x1p-46f);
    return {__uint_as_float(hb), l};
}

// a.h * b.h exactly plus the first-order cross terms: p + e ~ a * b (2^-46)
__device__ __forceinline__ dfl df_prod(dfl a, dfl b)
{
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return {p, e};
}

// a + b for unnormalised pairs (TwoSum of the high parts)
__device__ __forceinline__ dfl df_sum(dfl a, dfl b)
{
    const dfl s = df_two_sum(a.h, b.h);
    return {s.h, s.l + (a.l + b.l)};
}

// 1 / s as a float pair: rcp.approx seed, one Newton step on the pair's
// residual (relative error ~2^-46); 1/inf = 0
__device__ __forceinline__ dfl df_recip(dfl s)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s.h));
    float e = fmaf(-s.h, r, 1.0f);
    e = fmaf(-s.l, r, e);
    return {r, r == 0.0f ? 0.0f : r * e};
}

// ---------------------------------------------------------------- status
__device__ __forceinline__ void flag(int *status, int bit)
{
    if (status) atomicOr(status, bit);
}

}  // namespace gbx
