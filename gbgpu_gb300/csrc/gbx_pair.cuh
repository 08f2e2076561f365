// Pair form of the waveform family: the slow part, the N-point FFTs and the
// inner product <d|h> in float-pair arithmetic on the FP32 pipe.
//
// A value is the unevaluated sum h + l of two FP32 numbers (Dekker 1971;
// error-free TwoSum, Knuth TAOCP vol. 2, 4.2.2, and TwoProd through FMA), so
// sums and products keep about 44 significant bits while every instruction
// runs on the FP32 pipe (on GB300 one FP64 instruction takes the issue time
// of 64 FP32 ones).  An FP32 template carries ~1e-7 relative error, and in
// crowded data (a window 10-100x louder than the template) that error meets
// the loud bins: an FP32-valued template misses |dlogL| <= 1e-6 max(1, <h|h>)
// there even when rounded once from exact values.  The pair template carries
// ~1e-11 and the likelihood's <d|h> and <h|h> are summed in pairs, so every
// output stays within ~1e-9 of the FP64 form.
//
// This file is included inside namespace gbx by gbx_wave.cu.

// ---------------------------------------------------------------- arithmetic
// p_ sums are renormalised (Fast2Sum of head and tail): after a cancellation
// the tail of an unnormalised sum can reach the size of its head, and a later
// product would then round its cross term on that tail to FP32 precision
// relative to the (small) result; the u_ forms below skip it where that does
// not matter.  Products are not renormalised: their tail is the exact
// rounding error of the head plus the operands' cross terms, within a few
// units in the last place of the head, so the next operation keeps ~44
// significant bits without the three instructions of a renormalisation.
__device__ __forceinline__ dfl p_add(dfl a, dfl b) { return df_add(a, b); }
__device__ __forceinline__ dfl p_sub(dfl a, dfl b) { return p_add(a, dfl{-b.h, -b.l}); }

// a + b when |a.h| >= |b.h| (or a = 0): Fast2Sum of the heads, renormalised
__device__ __forceinline__ dfl p_addf(dfl a, dfl b)
{
    const float s = a.h + b.h;
    return df_fast(s, (b.h - (s - a.h)) + (a.l + b.l));
}

__device__ __forceinline__ dfl p_mul(dfl a, dfl b)
{
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return {p, e};
}

__device__ __forceinline__ dfl p_mulf(dfl a, float b)
{
    const float p = a.h * b;
    return {p, fmaf(a.l, b, fmaf(a.h, b, -p))};
}

__device__ __forceinline__ dfl p_scale(dfl a, float pow2) { return dfl{a.h * pow2, a.l * pow2}; }

__device__ __forceinline__ dfl p_sqr(dfl a)
{
    const float p = a.h * a.h;
    return {p, fmaf(a.h + a.h, a.l, fmaf(a.h, a.h, -p))};
}

// a b + c d
__device__ __forceinline__ dfl p_dot2(dfl a, dfl b, dfl c, dfl d)
{
    const float p = a.h * b.h, q = c.h * d.h;
    float e = fmaf(a.h, b.h, -p);
    float f = fmaf(c.h, d.h, -q);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    f = fmaf(c.h, d.l, fmaf(c.l, d.h, f));
    const dfl s = df_two_sum(p, q);
    return df_fast(s.h, s.l + (e + f));
}

// a b + c d + e f
__device__ __forceinline__ dfl p_dot3(dfl a, dfl b, dfl c, dfl d, dfl e, dfl f)
{
    const float p = a.h * b.h, q = c.h * d.h, r = e.h * f.h;
    float ep = fmaf(a.h, b.h, -p), eq = fmaf(c.h, d.h, -q), er = fmaf(e.h, f.h, -r);
    ep = fmaf(a.h, b.l, fmaf(a.l, b.h, ep));
    eq = fmaf(c.h, d.l, fmaf(c.l, d.h, eq));
    er = fmaf(e.h, f.l, fmaf(e.l, f.h, er));
    const dfl s1 = df_two_sum(p, q);
    const dfl s2 = df_two_sum(s1.h, r);
    return df_fast(s2.h, (s1.l + s2.l) + (ep + (eq + er)));
}

// n / d (FP32 quotient of the heads, one correction from the pair residual)
__device__ __forceinline__ dfl p_div(dfl n, dfl d)
{
    const float q1 = n.h / d.h;
    const dfl r = p_sub(n, p_mulf(d, q1));
    return df_fast(q1, (r.h + r.l) / d.h);
}

__device__ __forceinline__ cpx cp_add(cpx a, cpx b) { return {p_add(a.x, b.x), p_add(a.y, b.y)}; }
__device__ __forceinline__ cpx cp_sub(cpx a, cpx b) { return {p_sub(a.x, b.x), p_sub(a.y, b.y)}; }
__device__ __forceinline__ cpx cp_pow2(cpx a, float s) { return {p_scale(a.x, s), p_scale(a.y, s)}; }
__device__ __forceinline__ cpx cp_mul(cpx a, cpx b)
{
    return {p_dot2(a.x, b.x, df_neg(a.y), b.y), p_dot2(a.x, b.y, a.y, b.x)};
}
__device__ __forceinline__ cpx cp_scale(cpx a, dfl r) { return {p_mul(a.x, r), p_mul(a.y, r)}; }
__device__ __forceinline__ cpx cp_zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }

// Where an operation's error is judged against the size of its inputs (the
// transform's butterflies, the TDI combination, the projections and
// antenna patterns, series and link angles) the renormalisation adds
// nothing: after a cancellation the unnormalised tail is at most a few units
// in the last place of the INPUTS' heads, so the FP32 rounding of the later
// tail additions and cross terms stays below 2^-48 of the input size, the
// error the inputs already carry.  These u_ forms keep TwoSum's exact error
// and skip the closing Fast2Sum (3 of 11 instructions).  Sums stay
// renormalised where a head alone is read: the carrier phase before its
// reduction mod 2 pi (a phase of 1e3 rad would leave a tail of 1e-4 rad,
// and sincos picks its table entry from the head) and sincos's outputs.
__device__ __forceinline__ dfl u_add(dfl a, dfl b)
{
    const dfl s = df_two_sum(a.h, b.h);
    return {s.h, s.l + (a.l + b.l)};
}
__device__ __forceinline__ dfl u_sub(dfl a, dfl b) { return u_add(a, dfl{-b.h, -b.l}); }
__device__ __forceinline__ dfl u_dot2(dfl a, dfl b, dfl c, dfl d)
{
    const float p = a.h * b.h, q = c.h * d.h;
    float e = fmaf(a.h, b.h, -p);
    float f = fmaf(c.h, d.h, -q);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    f = fmaf(c.h, d.l, fmaf(c.l, d.h, f));
    const dfl s = df_two_sum(p, q);
    return {s.h, s.l + (e + f)};
}
// a b + c d + e f, unnormalised
__device__ __forceinline__ dfl u_dot3(dfl a, dfl b, dfl c, dfl d, dfl e, dfl f)
{
    const float p = a.h * b.h, q = c.h * d.h, r = e.h * f.h;
    float ep = fmaf(a.h, b.h, -p), eq = fmaf(c.h, d.h, -q), er = fmaf(e.h, f.h, -r);
    ep = fmaf(a.h, b.l, fmaf(a.l, b.h, ep));
    eq = fmaf(c.h, d.l, fmaf(c.l, d.h, eq));
    er = fmaf(e.h, f.l, fmaf(e.l, f.h, er));
    const dfl s1 = df_two_sum(p, q);
    const dfl s2 = df_two_sum(s1.h, r);
    return {s2.h, (s1.l + s2.l) + (ep + (eq + er))};
}
// a + b when |a.h| >= |b.h| (or a = 0), unnormalised
__device__ __forceinline__ dfl u_addf(dfl a, dfl b)
{
    const float s = a.h + b.h;
    return {s, (b.h - (s - a.h)) + (a.l + b.l)};
}
__device__ __forceinline__ cpx cu_add(cpx a, cpx b) { return {u_add(a.x, b.x), u_add(a.y, b.y)}; }
__device__ __forceinline__ cpx cu_sub(cpx a, cpx b) { return {u_sub(a.x, b.x), u_sub(a.y, b.y)}; }
__device__ __forceinline__ cpx cu_mul(cpx a, cpx b)
{
    return {u_dot2(a.x, b.x, df_neg(a.y), b.y), u_dot2(a.x, b.y, a.y, b.x)};
}
__device__ __forceinline__ double pd(dfl a) { return (double)a.h + (double)a.l; }

// ---------------------------------------------------------------- functions
// cos x and sin x for a pair |x| < 100 from a table of the pairs cos, sin at
// j pi/128 (tab[j & 255]) and the Taylor series on the remainder |d| <= pi/256:
// sin d = d - d^3/6 (next term below 3e-12), cos d = 1 - d^2/2 + d^4/24
// (below 5e-15), combined by the angle-addition formulas.  pi/128 = C1 + C2
// + C3 with C1 of 12 significant bits, so j C1 is exact for |j| < 4096 and
// x.h - j C1 is formed exactly by TwoSum.
constexpr int kScN = 256;

__device__ __forceinline__ void sincos_pair(dfl x, const float4 *__restrict__ tab, dfl &c, dfl &s)
{
    constexpr float kInv = 40.743663787841797f;     // 128/pi (picks j only)
    constexpr float C1 = 0.02454376220703125f;     // 3217 * 2^-17
    constexpr float C2 = -6.960085841001273e-08f;
    constexpr float C3 = -2.581268532253489e-15f;
    const float jf = rintf(x.h * kInv);
    const dfl h = df_two_sum(x.h, -jf * C1);
    const dfl d = df_fast(h.h, h.l + fmaf(-jf, C3, fmaf(-jf, C2, x.l)));
    const float4 t = tab[(int)jf & (kScN - 1)];
    const float d2 = d.h * d.h;
    const dfl sd = {d.h, fmaf(d.h * d2, -1.0f / 6.0f, d.l)};
    const float eps = d2 * fmaf(d2, 1.0f / 24.0f, -0.5f);   // cos d - 1
    const dfl Tc = {t.x, t.y}, Ts = {t.z, t.w};
    const dfl cc = u_add(Tc, df_neg(p_mul(Ts, sd)));
    const dfl ss = u_add(Ts, p_mul(Tc, sd));
    c = df_fast(cc.h, fmaf(Tc.h, eps, cc.l));
    s = df_fast(ss.h, fmaf(Ts.h, eps, ss.l));
}

// sincos_pair to ~1e-13 absolute, for angles whose sine enters a small
// factor relative to its own size (omL ~ 1e-2 in the TDI factors): the
// d^5 term of sin d, cos d - 1 = -d^2/2 + d^4/24 - d^6/720 as a pair with
// the d.l cross term, and pair products of the table values with it.
__device__ __forceinline__ void sincos_pair_acc(dfl x, const float4 *__restrict__ tab, dfl &c, dfl &s)
{
    constexpr float kInv = 40.743663787841797f;
    constexpr float C1 = 0.02454376220703125f;
    constexpr float C2 = -6.960085841001273e-08f;
    constexpr float C3 = -2.581268532253489e-15f;
    const float jf = rintf(x.h * kInv);
    const dfl h = df_two_sum(x.h, -jf * C1);
    const dfl d = df_fast(h.h, h.l + fmaf(-jf, C3, fmaf(-jf, C2, x.l)));
    const float4 t = tab[(int)jf & (kScN - 1)];
    const float d2 = d.h * d.h;
    const float d2l = fmaf(d.h + d.h, d.l, fmaf(d.h, d.h, -d2));
    const dfl sd = df_fast(d.h, fmaf(d.h * d2, fmaf(d2, 1.0f / 120.0f, -1.0f / 6.0f), d.l));
    const dfl em = df_fast(-0.5f * d2, fmaf(d2 * d2, fmaf(d2, -1.0f / 720.0f, 1.0f / 24.0f),
                                            -0.5f * d2l));
    const dfl Tc = {t.x, t.y}, Ts = {t.z, t.w};
    c = p_add(u_add(Tc, p_mul(Tc, em)), df_neg(p_mul(Ts, sd)));
    s = p_add(u_add(Ts, p_mul(Ts, em)), p_mul(Tc, sd));
}

// sin(a)/a alone: the S half of sinc_cos_pair.
__device__ __forceinline__ dfl sinc_pair(dfl a, const float4 *__restrict__ tab)
{
    const dfl x = p_sqr(a);
    const float xf = x.h;
    if (xf < 2.56f) {
        constexpr dfl s2 = dconst(1.0 / 120.0), s1 = dconst(-1.0 / 6.0);
        float q = fmaf(xf, -1.0f / 1307674368000.0f, 1.0f / 6227020800.0f);
        q = fmaf(q, xf, -1.0f / 39916800.0f);
        q = fmaf(q, xf, 1.0f / 362880.0f);
        q = fmaf(q, xf, -1.0f / 5040.0f);
        dfl r = u_addf(s2, dfl{xf * q, 0.f});
        r = u_addf(s1, p_mul(x, r));
        return u_addf(dfl{1.f, 0.f}, p_mul(x, r));
    }
    dfl c, sn;
    sincos_pair(a, tab, c, sn);
    return p_div(sn, a);
}

// sin(a)/a and cos(a) for a pair a >= 0: Taylor series in x = a^2 for
// x < 2.56 (terms to x^7; truncation below 5e-12 and 9e-11), the leading three
// coefficients as pairs and the rest as an FP32 tail (at most 4e-10 of the
// result); beyond that cos and sin from sincos_pair and one pair division.
__device__ __forceinline__ void sinc_cos_pair(dfl a, const float4 *__restrict__ tab, dfl &S, dfl &C)
{
    const dfl x = p_sqr(a);
    const float xf = x.h;
    if (xf < 2.56f) {
        constexpr dfl s2 = dconst(1.0 / 120.0), s1 = dconst(-1.0 / 6.0);
        float q = fmaf(xf, -1.0f / 1307674368000.0f, 1.0f / 6227020800.0f);
        q = fmaf(q, xf, -1.0f / 39916800.0f);
        q = fmaf(q, xf, 1.0f / 362880.0f);
        q = fmaf(q, xf, -1.0f / 5040.0f);
        dfl r = p_addf(s2, dfl{xf * q, 0.f});
        r = p_addf(s1, p_mul(x, r));
        S = p_addf(dfl{1.f, 0.f}, p_mul(x, r));
        constexpr dfl c2 = dconst(1.0 / 24.0);
        float u = fmaf(xf, -1.0f / 87178291200.0f, 1.0f / 479001600.0f);
        u = fmaf(u, xf, -1.0f / 3628800.0f);
        u = fmaf(u, xf, 1.0f / 40320.0f);
        u = fmaf(u, xf, -1.0f / 720.0f);
        dfl v = p_addf(c2, dfl{xf * u, 0.f});
        v = p_addf(dfl{-0.5f, 0.f}, p_mul(x, v));
        C = p_add(dfl{1.f, 0.f}, p_mul(x, v));
    } else {
        dfl sn;
        sincos_pair(a, tab, C, sn);
        S = p_div(sn, a);
    }
}

// ---------------------------------------------------------------- unequal arms
// slow_unequal_fp64 (gbx_wave.cu) in pair arithmetic: arm lengths ell_a L
// with ell_a = |r_a|, per-link transfer argument (f/f*)(ell_a +- k.r_a)/2,
// antenna pattern over ell_a, delays D_a = exp(-i x_a), x_a = omL ell_a, and
//   X = -2i omL [(1 - D_31^2)(G21 + D_12 G12) - (1 - D_12^2)(G31 + D_31 G13)]
// (Y, Z cyclic; TDI-2: times 1 - D_12^2 D_31^2, cyclic).  The small factors
// are formed without cancellation, 1 - e^{-2ix} = 2i sin(x) e^{-ix}, so
//   X = 4 omL [s_31 D_31 (G21 + D_12 G12) - s_12 D_12 (G31 + D_31 G13)]
// with s_a = sin x_a, and the TDI-2 factor is 2i sin(x_12 + x_31) D_12 D_31.
// A[] holds the arm patterns r.e.r / 4, E[] the spacecraft carriers, fo[]
// f/f* per spacecraft.
__device__ __forceinline__ cpx cp_mul_2i(cpx z) { return {p_scale(z.y, -2.f), p_scale(z.x, 2.f)}; }

template <bool AE>
__device__ __forceinline__ void slow_pair_unequal(const dfl (&r)[3][3], const dfl (&kr)[3],
                                               const dfl (&fo)[3], const cpx (&E)[3],
                                               const cpx (&A0)[3], dfl omL, int tdi,
                                               const float4 *__restrict__ sct, cpx out[3])
{
    dfl ell[3];
    cpx A[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const dfl e2 = p_dot3(r[a][0], r[a][0], r[a][1], r[a][1], r[a][2], r[a][2]);
        const float sq = sqrtf(e2.h);
        ell[a] = df_fast(sq, (fmaf(-sq, sq, e2.h) + e2.l) * (0.5f / sq));
        A[a] = cp_scale(A0[a], df_recip(ell[a]));
    }
    cpx G[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const int arm = q < 3 ? q : q - 3;
        const int s = q < 3 ? q : (q - 2) % 3;
        const dfl k = q < 3 ? kr[arm] : df_neg(kr[arm]);
        const dfl a = p_scale(p_mul(fo[s], p_addf(ell[arm], k)), 0.5f);
        dfl S, C;
        sinc_cos_pair(a, sct, S, C);
        const cpx T = {p_mul(S, C), df_neg(p_mul(p_mul(a, S), S))};
        G[q] = cp_mul(cp_mul(T, A[arm]), E[s]);
    }
    cpx D[3];
    dfl sn[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        dfl c;
        sincos_pair_acc(p_mul(omL, ell[a]), sct, c, sn[a]);
        D[a] = {c, df_neg(sn[a])};
    }
    // s_a D_a (G_q1 + D_b G_q2)
    auto term = [&](int a, int b, int q1, int q2) {
        return cp_scale(cp_mul(D[a], cp_add(G[q1], cp_mul(D[b], G[q2]))), sn[a]);
    };
    cpx X = cp_sub(term(2, 0, 3, 0), term(0, 2, 2, 5));
    cpx Y = cp_sub(term(0, 1, 4, 1), term(1, 0, 0, 3));
    cpx Z = cp_sub(term(1, 2, 5, 2), term(2, 1, 1, 4));
    if (tdi & GBX_TDI2_BIT) {
        // 2i sin(x_a + x_b) D_a D_b
        auto fac = [&](int a, int b) {
            const dfl sab = p_dot2(sn[a], D[b].x, D[a].x, sn[b]);
            return cp_mul_2i(cp_scale(cp_mul(D[a], D[b]), sab));
        };
        X = cp_mul(fac(0, 2), X);
        Y = cp_mul(fac(1, 0), Y);
        Z = cp_mul(fac(2, 1), Z);
    }
    const dfl w = p_scale(omL, 4.f);
    X = cp_scale(X, w);
    Y = cp_scale(Y, w);
    Z = cp_scale(Z, w);
    if constexpr (AE) {
        out[0] = cp_scale(cp_sub(Z, X), dconst(0.70710678118654752440));
        out[1] = cp_scale(cp_add(cp_sub(X, cp_pow2(Y, 2.f)), Z), dconst(0.40824829046386301637));
    } else {
        out[0] = X;
        out[1] = Y;
        out[2] = Z;
    }
}

// ---------------------------------------------------------------- slow part
// The slow part at one sample (gbgpu.py:399-540 and 348-375), as slow_mixed
// but every quantity a pair.  AE: out[0], out[1] = A, E (formed before the
// transform); otherwise out[0..2] = X, Y, Z.  Amplitude divided out.
//
// Each link carries its spacecraft's carrier in one exponential:
//   G_q = sinc(a_q) exp(-i (a_q + phi_s)) A_arm / 4
// (one sincos of the summed angle instead of exp(-i a_q) times
// exp(-i phi_s)), and with X' = G21 - G31, D_1 = G12 - G13 (cyclic) the TDI
// combination X = fc2 (X' + fc D_1) (gbgpu.py:370-375) gives
//   A = fc2/sqrt2 [(Z' - X') + fc (D_3 - D_1)],
//   E = fc2/sqrt6 [(X' - 2Y' + Z') + fc (D_1 - 2 D_2 + D_3)]:
// four complex products for A and E.
template <bool AE, bool UNEQ>
__device__ __forceinline__ void slow_pair(const Bin &B, int n, int N, dfl step, dfl Loc,
                                          const double *__restrict__ tab,
                                          const float4 *__restrict__ sct, cpx out[3], int tdi)
{
    const float *tabf = reinterpret_cast<const float *>(tab + (size_t)18 * N);
    // arm vectors r_12, r_23, r_31 = (P_j - P_i)/L close (sum to zero to
    // ~1e-14): with equal arms, arm 3's projections are minus the sum of the
    // other two; the unequal-arm model reads all three (it needs |r_a|)
    constexpr int NA = UNEQ ? 3 : 2;
    dfl r[3][3];
#pragma unroll
    for (int a = 0; a < NA; a++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            r[a][c] = {__ldg(tabf + (size_t)(3 * a + c) * N + n),
                       __ldg(tabf + (size_t)(27 + 3 * a + c) * N + n)};
    dfl kr[3];
#pragma unroll
    for (int a = 0; a < NA; a++)
        kr[a] = u_dot3(B.kd[0], r[a][0], B.kd[1], r[a][1], B.kd[2], r[a][2]);
    if constexpr (!UNEQ) kr[2] = df_neg(u_add(kr[0], kr[1]));
    const dfl tm = p_mulf(step, (float)n);                 // n T/N
    const float tf = tm.h;
    const dfl tm2 = p_sqr(tm);
    // carrier phase of spacecraft 1 (the expansion in slow_mixed):
    //   Phi0(tm) + kP w(tm) - pi kP^2 fd(tm) + pi/3 fddot kP^3
    dfl Phi0 = p_add(p_mul(B.omdfad, tm), B.phi0d);
    Phi0 = df_neg(p_add(Phi0, p_mul(tm2, p_add(B.pfd, p_mul(B.p3d, tm)))));
    const dfl wt = p_add(B.omd, p_add(p_mul(B.tpfd, tm), p_mul(B.pfddd, tm2)));
    const float fdt = fmaf(B.fddotf, tf, B.fdotf);
    const dfl kP0 = kP1_pair(B, tabf, N, n);
    dfl ph0 = p_add(Phi0, p_mul(kP0, wt));
    {
        const float q = rintf(ph0.h * (float)kInvTwoPi);
        ph0 = p_add(ph0, df_neg(p_mulf(dconst(kTwoPi), q)));
    }
    // spacecraft 2 and 3: k.P_s/c = k.P_1/c + (L/c) k.r_12 and - (L/c) k.r_31
    const dfl dk[3] = {dfl{0.f, 0.f}, p_mul(Loc, kr[0]), df_neg(p_mul(Loc, kr[2]))};
    // f(t)/fstar = w0 + w1 t + w2 t^2 with w1 t a pair: at f0 = 1e-4 Hz and
    // fdot = 1e-15 that term is 1e-3 of w0, and omL enters fc2 squared
    const dfl base = u_addf(dfl{B.w0h, B.w0l}, p_mul(dfl{B.w1, B.w1l}, tm));
    cpx E[3];
    dfl fo[3], phs[3];
#pragma unroll
    for (int s = 0; s < 3; s++) {
        dfl ph = s == 0 ? ph0 : p_add(ph0, p_mul(dk[s], wt));
        const float kPf = kP0.h + dk[s].h;
        ph.l += kPf * kPf * fmaf(kPf, B.p3d.h, -(float)kPi * fdt);   // below 1e-8 rad
        phs[s] = ph;
        if constexpr (UNEQ) {
            dfl cs, sn;
            sincos_pair(ph, sct, cs, sn);
            E[s] = {cs, df_neg(sn)};
        }
        // f(xi)/fstar at xi = t - kP: - w1 kP + w2 xi^2 are below 3e-6 of w0
        const float xf = tf - kPf;
        fo[s] = u_addf(base, dfl{fmaf(B.w2 * xf, xf, -B.w1 * kPf), 0.f});
    }
    // antenna patterns per arm, with the 1/4 of the transfer functions:
    // r.e+.r = (r.v)^2 - (r.u)^2, r.ex.r = 2 (r.u)(r.v)
    cpx A[3];
    dfl rus[2], rvs[2];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        dfl ru, rv;
        if (a < NA) {
            ru = u_dot3(B.pr.ud[0], r[a][0], B.pr.ud[1], r[a][1], B.pr.ud[2], r[a][2]);
            rv = u_dot2(B.pr.vd[0], r[a][0], B.pr.vd[1], r[a][1]);
        } else {
            ru = df_neg(u_add(rus[0], rus[1]));
            rv = df_neg(u_add(rvs[0], rvs[1]));
        }
        if (a < 2) {
            rus[a] = ru;
            rvs[a] = rv;
        }
        const dfl pp = p_scale(u_dot2(rv, rv, df_neg(ru), ru), 0.25f);
        const dfl cc = p_scale(p_mul(ru, rv), 0.5f);
        A[a] = {u_dot2(pp, B.pr.DP.x, cc, B.pr.DC.x), u_dot2(pp, B.pr.DP.y, cc, B.pr.DC.y)};
    }
    if constexpr (UNEQ) {
        slow_pair_unequal<AE>(r, kr, fo, E, A, p_addf(base, dfl{B.w2 * tf * tf, 0.f}), tdi, sct, out);
        return;
    }
    // links (ij, arm, spacecraft): 12,23,31 (+k.r) and 21,32,13 (-k.r); the two
    // links of arm a (spacecraft a and a+1) carry angles th+ = a+ + phi_a and
    // th- = a- + phi_(a+1) that differ by
    //   d = (fo_(a+1) - fo_a)/2 + k.r (f(t)/f* - (fo_a + fo_(a+1))/2) + (k.P^2 terms),
    // |d| < 1e-7 rad (fdot k.P/f* and the phase's k.P^2 terms), so
    // exp(-i th-) A_a = exp(-i th+) A_a (1 - i d) to 1e-14: one pair sincos
    // and one complex product per arm.  (|d| >= 1e-4 would take the full
    // sincos; it does not occur for equal arms.)
    cpx G[6];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int s2 = a == 2 ? 0 : a + 1;
        const dfl ap = p_scale(p_mul(fo[a], p_addf(dfl{1.f, 0.f}, kr[a])), 0.5f);
        const dfl am = p_scale(p_mul(fo[s2], p_addf(dfl{1.f, 0.f}, df_neg(kr[a]))), 0.5f);
        const dfl Sp = sinc_pair(ap, sct), Sm = sinc_pair(am, sct);
        const dfl thp = u_add(ap, phs[a]), thm = u_add(am, phs[s2]);
        dfl c, sn;
        sincos_pair(thp, sct, c, sn);
        const cpx eA = cu_mul(cpx{c, df_neg(sn)}, A[a]);
        G[a] = {p_mul(Sp, eA.x), p_mul(Sp, eA.y)};
        const dfl dl = u_sub(thm, thp);
        const float d = dl.h + dl.l;
        cpx eAm;
        if (fabsf(d) < 1e-4f) {
            eAm = {u_add(eA.x, dfl{d * eA.y.h, 0.f}), u_add(eA.y, dfl{-d * eA.x.h, 0.f})};
        } else {
            sincos_pair(thm, sct, c, sn);
            eAm = cu_mul(cpx{c, df_neg(sn)}, A[a]);
        }
        G[a + 3] = {p_mul(Sm, eAm.x), p_mul(Sm, eAm.y)};
    }
    // omega L, fc = e^{-i omL}, fc2 = 4 omL sin(omL) fc (gbgpu.py:362-368)
    const dfl omL = u_addf(base, dfl{B.w2 * tf * tf, 0.f});
    dfl co, so;
    sincos_pair_acc(omL, sct, co, so);   // sin(omL) scales the window: relative accuracy at low f
    const cpx fc = {co, df_neg(so)};
    const dfl g4 = p_scale(p_mul(omL, so), 4.f);
    if constexpr (AE) {
        // A = (Z - X)/sqrt2, E = (X - 2Y + Z)/sqrt6 (utility.py:24-38), with
        //   Z' - X' = (G31 + G13) - (G23 + G21),  D3 - D1 = (G31 + G13) - (G12 + G32),
        //   X' - 2Y' + Z' = 2 (G12 - G32) + (G21 - G23) + (G13 - G31),
        //   D1 - 2 D2 + D3 = (G12 - G32) + 2 (G21 - G23) - (G13 - G31)
        const cpx s25 = cu_add(G[2], G[5]);
        const cpx ga = cu_sub(G[0], G[4]), gb = cu_sub(G[3], G[1]), gc = cu_sub(G[5], G[2]);
        const cpx wA = cu_add(cu_sub(s25, cu_add(G[1], G[3])),
                              cu_mul(fc, cu_sub(s25, cu_add(G[0], G[4]))));
        const cpx wE = cu_add(cu_add(cp_pow2(ga, 2.f), cu_add(gb, gc)),
                              cu_mul(fc, cu_sub(cu_add(ga, cp_pow2(gb, 2.f)), gc)));
        const dfl gA = p_mul(g4, dconst(0.70710678118654752440));
        const dfl gE = p_mul(g4, dconst(0.40824829046386301637));
        out[0] = cu_mul(cpx{p_mul(gA, co), df_neg(p_mul(gA, so))}, wA);
        out[1] = cu_mul(cpx{p_mul(gE, co), df_neg(p_mul(gE, so))}, wE);
    } else {
        const cpx D1 = cu_sub(G[0], G[5]), D2 = cu_sub(G[1], G[3]), D3 = cu_sub(G[2], G[4]);
        const cpx X0 = cu_sub(G[3], G[2]), Y0 = cu_sub(G[4], G[0]), Z0 = cu_sub(G[5], G[1]);
        const cpx fc2 = {p_mul(g4, co), df_neg(p_mul(g4, so))};
        out[0] = cu_mul(fc2, cu_add(X0, cu_mul(fc, D1)));
        out[1] = cu_mul(fc2, cu_add(Y0, cu_mul(fc, D2)));
        out[2] = cu_mul(fc2, cu_add(Z0, cu_mul(fc, D3)));
    }
}

// ---------------------------------------------------------------- FFT
// fft_dif in pair arithmetic: same passes, swizzle and output order; the
// twiddles are pairs of the FP64 table.
__device__ __forceinline__ cpx tw_pair(int m)
{
    const float4 t = g_tw_p[m];
    return {{t.x, t.y}, {t.z, t.w}};
}

template <int RB>
__device__ __forceinline__ void fft_reg_pass_pair(cpx *buf, int nsub, int lg, int hl)
{
    constexpr int M = 1 << RB;
    const int q = hl - RB + 1;
    const int groups = nsub << (lg - RB);
    for (int g = threadIdx.x; g < groups; g += kBlock) {
        const int a = g >> (lg - RB);
        const int rem = g & ((1 << (lg - RB)) - 1);
        const int blk = rem >> q;
        const int r = rem & ((1 << q) - 1);
        cpx *sub = buf + ((size_t)a << lg);
        const int p0 = (blk << (hl + 1)) + r;
        cpx x[M];
#pragma unroll
        for (int m = 0; m < M; m++) x[m] = sub[swz(p0 + (m << q), lg)];
#pragma unroll
        for (int j = 0; j < RB; j++) {
            const int dm = M >> (j + 1);
            const int hh = hl - j;
            const int ts = kTwN >> (hh + 1);
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (m & dm) continue;
                const int rp = r + ((m & (dm - 1)) << q);
                const cpx u = x[m], v = x[m + dm];
                x[m] = cu_add(u, v);
                x[m + dm] = cu_mul(cu_sub(u, v), tw_pair(rp * ts));
            }
        }
#pragma unroll
        for (int m = 0; m < M; m++) sub[swz(p0 + (m << q), lg)] = x[m];
    }
}

__device__ __forceinline__ float shfl4(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }

__device__ __forceinline__ void fft_dif_pair(cpx *buf, int nsub, int lg)
{
    int hl = lg - 1;
    while (hl >= 5) {
        const int rb = (hl - 4) >= 3 ? 3 : (hl - 4);
        if (rb == 3) fft_reg_pass_pair<3>(buf, nsub, lg, hl);
        else if (rb == 2) fft_reg_pass_pair<2>(buf, nsub, lg, hl);
        else fft_reg_pass_pair<1>(buf, nsub, lg, hl);
        hl -= rb;
        __syncthreads();
    }
    // Last five stages (half-spans 16 ... 1) on 32-element blocks, one block
    // per half-warp, lane l holding two elements: first positions l and
    // l + 16 (the span-16 butterfly in registers), then before each later
    // stage of half-span h the lane trades one element with lane l ^ h so
    // that it holds the pair (e, e + h) of the in-place transform (e = l mod
    // h plus multiples of 2h), and ends with positions 2l, 2l + 1.  Same
    // operations and operand order as stage-by-stage butterflies, two
    // elements per lane: no butterfly is computed twice.
    const int lane = threadIdx.x & 31;
    const int l = lane & 15;
    // half-span 2 takes W^0 = 1 and W^(kTwN/4) = -i (sincospi is exact
    // there): a swap and a sign instead of a product, with the same result
    cpx w[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int hh = 4 - k;
        w[k] = tw_pair((l & ((1 << hh) - 1)) * (kTwN >> (hh + 1)));
    }
    const int blocks = (nsub << lg) >> 5;
    const int npairs = (blocks + 1) >> 1;
    for (int c = threadIdx.x >> 5; c < npairs; c += kBlock >> 5) {
        const int blk = 2 * c + (lane >> 4);
        const bool live = blk < blocks;
        const int e0 = (live ? blk : blocks - 1) << 5;   // a spare half-warp repeats the last block
        cpx *sub = buf + ((e0 >> lg) << lg);
        const int off = e0 & ((1 << lg) - 1);
        cpx u = sub[swz(off + l, lg)], v = sub[swz(off + l + 16, lg)];
        {
            const cpx t = cu_sub(u, v);
            u = cu_add(u, v);
            v = cu_mul(t, w[0]);
        }
#pragma unroll
        for (int k = 1; k < 5; k++) {
            const int h = 16 >> k;
            const bool bit = (l & h) != 0;
            const cpx snd = bit ? u : v;
            const cpx rcv = {{shfl4(snd.x.h, h), shfl4(snd.x.l, h)}, {shfl4(snd.y.h, h), shfl4(snd.y.l, h)}};
            if (bit) u = rcv;
            else v = rcv;
            const cpx t = cu_sub(u, v);
            u = cu_add(u, v);
            if (k < 3) v = cu_mul(t, w[k]);
            else if (k == 3) v = (l & 1) ? cpx{t.y, df_neg(t.x)} : t;
            else v = t;
        }
        if (live) {
            sub[swz(off + 2 * l, lg)] = u;
            sub[swz(off + 2 * l + 1, lg)] = v;
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------- kernel
// One CTA per tile as wave_kernel; MODE_WAVE writes the reference's output
// arrays (the transformed pairs rounded once to FP64, then the FP64 scale
// and AET), MODE_LL folds the window into <d|h> and <h|h> (pairs).  Shared memory: the binaries' constants, the reduction
// scratch, the sin/cos table and the transform buffers.
template <int MODE, bool UNEQ>
__global__ void __launch_bounds__(kBlock, 2) pair_kernel(const KParams K)
{
    constexpr int NCH = MODE == MODE_WAVE ? 3 : 2;
    extern __shared__ __align__(16) unsigned char smem[];
    Bin *bins = reinterpret_cast<Bin *>(smem);
    double *red = reinterpret_cast<double *>(smem + sizeof(Bin) * K.maxP);
    float4 *sct = reinterpret_cast<float4 *>(smem + sizeof(Bin) * K.maxP +
                                             sizeof(double) * red_doubles(K.maxS));
    cpx *buf = reinterpret_cast<cpx *>(sct + kScN);
    __shared__ int s_tile;

    const gbx_wave_args &a = K.a;
    const int tid = threadIdx.x;
    for (int k = tid; k < kScN; k += kBlock) sct[k] = g_sc_p[k];
    const int ntiles = a.tiles ? a.ntiles : (a.num_bin + K.P - 1) / K.P;
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
        const double *tab = (lg >= 5 && lg <= kPairMaxLog2N)
                                ? reinterpret_cast<const double *>(a.orbit[lg]) : nullptr;
        const int maxcnt = tile_pack(a.tile, lg, MODE == MODE_SWAP ? 2 : 1);
        if (tab == nullptr || cnt < 1 || cnt > maxcnt || first < 0 || first + cnt > a.num_bin ||
            (cnt << lg) > K.maxS) {
            flag(a.status, GBX_FLAG_TILE);
            __syncthreads();
            continue;
        }
        if (a.workspace) {
            const int4 *src = reinterpret_cast<const int4 *>(static_cast<const Bin *>(a.workspace) + first);
            int4 *dst = reinterpret_cast<int4 *>(bins);
            const int n16 = cnt * (int)(sizeof(Bin) / 16);
            for (int k = tid; k < n16; k += kBlock) dst[k] = src[k];
        } else if (tid < cnt) {
            const int slot = first + tid;
            const int b = a.order ? a.order[slot] : slot;
            if (b < 0 || b >= a.num_bin) {
                flag(a.status, GBX_FLAG_TILE);
                memset(&bins[tid], 0, sizeof(Bin));
                bins[tid].b = -1;
            } else {
                setup_bin(bins[tid], K, b, N, MODE);
            }
        }
        __syncthreads();

        const int S = cnt << lg;
        const dfl stepd = K.stepd[lg];
        for (int m = tid; m < S; m += kBlock) {
            const int p = m >> lg, n = m & (N - 1);
            const Bin &B = bins[p];
            cpx o[3];
            if (!B.valid) {
                o[0] = o[1] = o[2] = cp_zero();
            } else {
                slow_pair<NCH == 2, UNEQ>(B, n, N, stepd, K.Locd, tab, sct, o, a.tdi2);
            }
#pragma unroll
            for (int c = 0; c < NCH; c++) buf[(p * NCH + c) * N + swz(n, lg)] = o[c];
        }
        __syncthreads();

        fft_dif_pair(buf, NCH * cnt, lg);

        if constexpr (MODE == MODE_WAVE) {
            for (int m = tid; m < S; m += kBlock) {
                const int p = m >> lg, i = m & (N - 1);
                const Bin &B = bins[p];
                if (B.b < 0) continue;
                const int pos = swz(bitrev((i + (N >> 1)) & (N - 1), lg), lg);   // fftshift
                const cpx X = buf[(p * 3 + 0) * N + pos], Y = buf[(p * 3 + 1) * N + pos],
                          Z = buf[(p * 3 + 2) * N + pos];
                const double2 Xd = cmul(make_double2(pd(X.x), pd(X.y)), B.scale);
                const double2 Yd = cmul(make_double2(pd(Y.x), pd(Y.y)), B.scale);
                const double2 Zd = cmul(make_double2(pd(Z.x), pd(Z.y)), B.scale);
                const size_t o = (size_t)B.b * 3 * N + i;
                if (K.XYZ) {
                    K.XYZ[o] = Xd;
                    K.XYZ[o + N] = Yd;
                    K.XYZ[o + 2 * N] = Zd;
                }
                if (K.AET) {
                    const double is2 = 0.70710678118654752440, is6 = 0.40824829046386301637;
                    const double i3 = 0.57735026918962576451;
                    K.AET[o] = make_double2((Zd.x - Xd.x) * is2, (Zd.y - Xd.y) * is2);
                    K.AET[o + N] = make_double2((Xd.x - 2.0 * Yd.x + Zd.x) * is6,
                                                (Xd.y - 2.0 * Yd.y + Zd.y) * is6);
                    K.AET[o + 2 * N] = make_double2((Xd.x + Yd.x + Zd.x) * i3, (Xd.y + Yd.y + Zd.y) * i3);
                }
                if (i == 0 && K.start_out) K.start_out[B.b] = B.start;
            }
        } else if constexpr (MODE == MODE_SWAP) {
            // as wave_kernel's MODE_SWAP: binaries 2j (current) and 2j+1
            // (proposal) of the tile form a pair, threads [j Tp2, (j+1) Tp2)
            // walk both windows; with r the residual row and Dh = h_new - h_old
            //   dlogL = Re<r|h_new> - Re<r|h_old> - (<h_new|h_new> + <h_old|h_old>)/2
            //           + Re<h_old|h_new>   (cross term on the windows' overlap),
            // every term summed in pairs
            const int Tp2 = 2 * (kBlock / maxcnt);
            const int width = Tp2 < 32 ? Tp2 : 32;
            const int pr = tid / Tp2;
            const int i0 = tid - pr * Tp2;
            const bool samepsd = K.A_psd == K.E_psd;
            dfl acc8[8];   // Crn (2), Cro (2), Hn, Ho, Cx (2)
#pragma unroll
            for (int k = 0; k < 8; k++) acc8[k] = dfl{0.f, 0.f};
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
                        const int pos = swz(bitrev((i + (N >> 1)) & (N - 1), lg), lg);
                        const cpx hA = buf[(pw * 2 + 0) * N + pos], hE = buf[(pw * 2 + 1) * N + pos];
                        const size_t jd = (size_t)Bn.di * K.L + j, jn = (size_t)Bn.ni * K.L + j;
                        const double2 dA = __ldg(K.A_data + jd), dE = __ldg(K.E_data + jd);
                        const dfl wA = df_recip(d2ff_scaled(__ldg(K.A_psd + jn), Bn.eS));
                        const dfl wE = samepsd ? wA : df_recip(d2ff_scaled(__ldg(K.E_psd + jn), Bn.eS));
                        const dfl ar = p_mul(d2ff_scaled(dA.x, Bn.eD), wA);
                        const dfl ai = p_mul(d2ff_scaled(dA.y, Bn.eD), wA);
                        const dfl er = p_mul(d2ff_scaled(dE.x, Bn.eD), wE);
                        const dfl ei = p_mul(d2ff_scaled(dE.y, Bn.eD), wE);
                        // conj(r) h / S and |h|^2 / S
                        const dfl cr = u_add(u_dot2(ar, hA.x, ai, hA.y), u_dot2(er, hE.x, ei, hE.y));
                        const dfl ci = u_add(u_dot2(ar, hA.y, df_neg(ai), hA.x),
                                             u_dot2(er, hE.y, df_neg(ei), hE.x));
                        const dfl hh2 = u_dot2(u_dot2(hA.x, hA.x, hA.y, hA.y), wA,
                                               u_dot2(hE.x, hE.x, hE.y, hE.y), wE);
                        if (isnew) {
                            acc8[0] = p_add(acc8[0], cr);
                            acc8[1] = p_add(acc8[1], ci);
                            acc8[4] = p_add(acc8[4], hh2);
                            const int k = j - Bo.start;
                            if (k >= 0 && k < N) {
                                const int pk = swz(bitrev((k + (N >> 1)) & (N - 1), lg), lg);
                                const cpx oA = buf[(po * 2 + 0) * N + pk], oE = buf[(po * 2 + 1) * N + pk];
                                // conj(h_old) h_new / S
                                acc8[6] = p_add(acc8[6], u_dot2(u_dot2(oA.x, hA.x, oA.y, hA.y), wA,
                                                                u_dot2(oE.x, hE.x, oE.y, hE.y), wE));
                                acc8[7] = p_add(acc8[7], u_dot2(u_dot2(oA.x, hA.y, df_neg(oA.y), hA.x), wA,
                                                                u_dot2(oE.x, hE.y, df_neg(oE.y), hE.x), wE));
                            }
                        } else {
                            acc8[2] = p_add(acc8[2], cr);
                            acc8[3] = p_add(acc8[3], ci);
                            acc8[5] = p_add(acc8[5], hh2);
                        }
                    }
                    if (out) flag(a.status, GBX_FLAG_WINDOW);
                }
            }
            {
                // group trees in pairs; the leaders write FP64 partials
                const bool leader = (tid & (width - 1)) == 0;
                const int g = tid / width;
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    dfl x = acc8[k];
                    for (int o = width >> 1; o > 0; o >>= 1)
                        x = p_add(x, dfl{shfl4(x.h, o), shfl4(x.l, o)});
                    if (leader) red[8 * g + k] = pd(x);
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
                const double cdh = 4.0 * K.df * exp2_int(Bn.eS - Bn.eD);
                const double chh = 4.0 * K.df * exp2_int(Bn.eS);
                const double2 so = Bo.scale, sn = Bn.scale;
                const double rn = cmul(sn, make_double2(t[0], t[1])).x * cdh;
                const double ro = cmul(so, make_double2(t[2], t[3])).x * cdh;
                const double hn = (sn.x * sn.x + sn.y * sn.y) * t[4] * chh;
                const double ho = (so.x * so.x + so.y * so.y) * t[5] * chh;
                const double cx = cmul(make_double2(so.x, -so.y), cmul(sn, make_double2(t[6], t[7]))).x * chh;
                const bool ok = Bo.valid && Bn.valid && Bo.b >= 0 && Bn.b >= 0;
                if (Bn.b >= 0) K.dlogl[Bn.b >> 1] = ok ? (rn - ro - 0.5 * (hn + ho) + cx) : 0.0;
            }
        } else if constexpr (MODE == MODE_FILL) {
            // as wave_kernel's MODE_FILL: each run of same-group binaries with
            // ascending, overlapping windows is summed once per bin of its span;
            // the pairs are rounded once to FP64 and scaled in FP64
            __shared__ int s_run[kMaxPack + 1], s_lo[kMaxPack], s_off[kMaxPack + 1];
            __shared__ int s_nruns;
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
                    const int pos = swz(bitrev((i + (N >> 1)) & (N - 1), lg), lg);
                    const cpx tA = buf[(p * 2 + 0) * N + pos], tE = buf[(p * 2 + 1) * N + pos];
                    const double2 a2 = cmul(make_double2(pd(tA.x), pd(tA.y)), B.scale);
                    const double2 e2 = cmul(make_double2(pd(tE.x), pd(tE.y)), B.scale);
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
        } else {
            // Threads [p Tpb, (p+1) Tpb) own binary p and stride its window (a
            // warp reads contiguous runs of data and PSD).  <d|h> and <h|h> per
            // thread and over lanes in pairs.
            const int Tpb = kBlock / maxcnt;
            const int width = Tpb < 32 ? Tpb : 32;
            const int p = tid / Tpb;
            const int i0 = tid - p * Tpb;
            dfl sr = {0.f, 0.f}, si = {0.f, 0.f}, xh = {0.f, 0.f};
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
                        const int pos = swz(bitrev((i + (N >> 1)) & (N - 1), lg), lg);
                        const cpx tA = buf[(p * 2 + 0) * N + pos], tE = buf[(p * 2 + 1) * N + pos];
                        const size_t jd = (size_t)B.di * K.L + j, jn = (size_t)B.ni * K.L + j;
                        const double2 dA = __ldg(K.A_data + jd), dE = __ldg(K.E_data + jd);
                        if (samepsd) {
                            // one PSD for both channels: the channels' terms summed, then
                            // one weight (gbgpu_utils.cu:172-178)
                            const dfl w = df_recip(d2ff_scaled(__ldg(K.A_psd + jn), B.eS));
                            const dfl ar = d2ff_scaled(dA.x, B.eD), ai = d2ff_scaled(dA.y, B.eD);
                            const dfl er = d2ff_scaled(dE.x, B.eD), ei = d2ff_scaled(dE.y, B.eD);
                            sr = p_add(sr, p_mul(u_add(u_dot2(ar, tA.x, ai, tA.y),
                                                       u_dot2(er, tE.x, ei, tE.y)), w));
                            si = p_add(si, p_mul(u_add(u_dot2(ar, tA.y, df_neg(ai), tA.x),
                                                       u_dot2(er, tE.y, df_neg(ei), tE.x)), w));
                            xh = p_add(xh, p_mul(u_add(u_dot2(tA.x, tA.x, tA.y, tA.y),
                                                       u_dot2(tE.x, tE.x, tE.y, tE.y)), w));
                        } else {
                            const dfl wA = df_recip(d2ff_scaled(__ldg(K.A_psd + jn), B.eS));
                            const dfl wE = df_recip(d2ff_scaled(__ldg(K.E_psd + jn), B.eS));
                            // conj(d) h / S  (gbgpu_utils.cu:172-178), d / S first
                            const dfl ar = p_mul(d2ff_scaled(dA.x, B.eD), wA);
                            const dfl ai = p_mul(d2ff_scaled(dA.y, B.eD), wA);
                            const dfl er = p_mul(d2ff_scaled(dE.x, B.eD), wE);
                            const dfl ei = p_mul(d2ff_scaled(dE.y, B.eD), wE);
                            sr = p_add(sr, u_add(u_dot2(ar, tA.x, ai, tA.y), u_dot2(er, tE.x, ei, tE.y)));
                            si = p_add(si, u_add(u_dot2(ar, tA.y, df_neg(ai), tA.x),
                                                   u_dot2(er, tE.y, df_neg(ei), tE.x)));
                            xh = p_add(xh, u_dot2(u_dot2(tA.x, tA.x, tA.y, tA.y), wA,
                                                   u_dot2(tE.x, tE.x, tE.y, tE.y), wE));
                        }
                    }
                }
                if (out) flag(a.status, GBX_FLAG_WINDOW);
            }
            for (int o = width >> 1; o > 0; o >>= 1) {
                sr = p_add(sr, dfl{shfl4(sr.h, o), shfl4(sr.l, o)});
                si = p_add(si, dfl{shfl4(si.h, o), shfl4(si.l, o)});
                xh = p_add(xh, dfl{shfl4(xh.h, o), shfl4(xh.l, o)});
            }
            if ((tid & (width - 1)) == 0) {
                float2 *red2 = reinterpret_cast<float2 *>(red);
                const int g = tid / width;
                red2[3 * g] = make_float2(sr.h, sr.l);
                red2[3 * g + 1] = make_float2(si.h, si.l);
                red2[3 * g + 2] = make_float2(xh.h, xh.l);
            }
            __syncthreads();
            double *tsum = red + 3 * kMaxPack;
            {
                const int per = Tpb / width;
                const float2 *red2 = reinterpret_cast<const float2 *>(red);
                for (int t = tid; t < 3 * cnt; t += kBlock) {
                    const int q = t / 3, c = t - 3 * q;
                    dfl x = {0.f, 0.f};
                    for (int g = q * per; g < (q + 1) * per; g++) {
                        const float2 y = red2[3 * g + c];
                        x = p_add(x, dfl{y.x, y.y});
                    }
                    tsum[t] = pd(x);
                }
            }
            __syncthreads();
            if (tid < cnt) {
                const Bin &B = bins[tid];
                const double s4 = 4.0 * K.df;
                const double cd = s4 * exp2_int(B.eS - B.eD);
                const double ch = s4 * exp2_int(B.eS) * (B.scale.x * B.scale.x + B.scale.y * B.scale.y);
                double2 dh = cmul(make_double2(cd * tsum[3 * tid], cd * tsum[3 * tid + 1]), B.scale);
                double2 hv = make_double2(ch * tsum[3 * tid + 2], 0.0);
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
