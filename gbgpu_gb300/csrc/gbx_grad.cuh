// Gradient of the log-likelihood with respect to the nine source parameters
// (amp, f0, fdot, fddot, phi0, iota, psi, lam, beta), fused with the
// likelihood itself.  Included by gbx_wave.cu (same translation unit: it uses
// the per-binary set-up, the slow part, the FFT and the twiddle tables).
//
// With r = d - h and w_c = the residual weights 4 df r / S mapped onto the
// X, Y, Z channels (A = (Z - X)/sqrt2, E = (X - 2Y + Z)/sqrt6):
//   d logL / d theta = Re sum_c sum_i conj(w_c,i) d h_c,i / d theta
//                    = Re[scale sum_c sum_n Y_c,n d x_c,n / d theta]
//                      + Re[(d scale / d theta) Qf],
// where x is the slow part (the reference's XYZsl, gbgpu.py:375), h = scale
// FFT(x) heterodyned (gbgpu.py:378-388), Y_c = DFT(conj(w_c)) (forward
// transform of the conjugated weights, which the kernel computes in place with
// a decimation-in-time FFT on the bit-reversed buffer), and
// Qf = sum conj(w) X.  The slow part is recomputed in the backward pass with
// analytic derivatives (nothing is stored between the passes).
//
// This file is included inside namespace gbx by gbx_wave.cu.

enum { MODE_GRAD = 3 };

struct __align__(16) GradExtra {
    float u[3], v[3];              // sky basis vectors (gbgpu.py:256-258)
    float st, ct;                  // sin / cos of the polar angle
    double2 dDPi, dDCi, dDPp, dDCp;  // d(DP, DC)/d(iota, psi), amplitude divided out
    double2 dlnsc_f0;              // d ln(scale) / d f0 (TDI-2 factor), 0 otherwise
    float gf0, gf1;                // d fonfs / d kP = -(fdot + fddot xi)/fstar = gf0 + gf1 xi
    float cosvarpi, P2yr;          // third body: cos varpi, period in years
};

__device__ void setup_grad(GradExtra &X, const KParams &K, int b)
{
    const gbx_wave_args &a = K.a;
    const int nb = a.num_bin;
    const double *p = a.params;
    double f0 = p[nb + b], fdot = p[2 * nb + b], fddot = p[3 * nb + b];
    double iota = p[5 * nb + b], psi = p[6 * nb + b], lam = p[7 * nb + b], beta = p[8 * nb + b];
    double theta = kPi / 2.0 - beta;
    double st, ct, sp, cp, si, ci, s2p, c2p;
    sincos(theta, &st, &ct);
    sincos(lam, &sp, &cp);
    sincos(iota, &si, &ci);
    sincos(2.0 * psi, &s2p, &c2p);
    X.u[0] = (float)(ct * cp); X.u[1] = (float)(ct * sp); X.u[2] = (float)(-st);
    X.v[0] = (float)sp; X.v[1] = (float)(-cp); X.v[2] = 0.0f;
    X.st = (float)st;
    X.ct = (float)ct;
    // DP = Ap c2p - i Ac s2p, DC = -Ap s2p - i Ac c2p; Ap = 1 + ci^2, Ac = -2 ci
    const double Ap = 1.0 + ci * ci, Ac = -2.0 * ci;
    const double dAp = -2.0 * ci * si, dAc = 2.0 * si;
    X.dDPi = make_double2(dAp * c2p, -dAc * s2p);
    X.dDCi = make_double2(-dAp * s2p, -dAc * c2p);
    X.dDPp = make_double2(-2.0 * Ap * s2p, -2.0 * Ac * c2p);
    X.dDCp = make_double2(-2.0 * Ap * c2p, 2.0 * Ac * s2p);
    X.dlnsc_f0 = make_double2(0.0, 0.0);
    if (a.tdi2) {
        // factor 2i sin(2wL) exp(-2iwL), wL = 2 pi f0 L/c: d ln/d f0 = (2 cot 2wL - 2i) 2 pi L/c
        const double c = 2.0 * kPi * (a.armlength / kCSI);
        const double wL = c * f0;
        X.dlnsc_f0 = make_double2(2.0 * c * cos(2.0 * wL) / sin(2.0 * wL), -2.0 * c);
    }
    X.gf0 = (float)(-fdot / K.fstar);
    X.gf1 = (float)(-fddot / K.fstar);
    X.cosvarpi = 0.0f;
    X.P2yr = 1.0f;
    if (a.nparams >= 14) {
        X.cosvarpi = (float)cos(p[10 * nb + b]);
        X.P2yr = (float)p[12 * nb + b];
    }
}

// S(a) = sin(a)/a, C = cos(a) and S'(a) from their Taylor series in x = a^2
// (|a| <= 1.6), library functions beyond.
__device__ __forceinline__ void sinc_cos_d_f(float a, float &S, float &C, float &dS)
{
    const float x = a * a;
    if (x < 2.56f) {
        sinc_cos_f(a, S, C);
        // S'(a) = a sum_{k>=1} (-1)^k 2k x^(k-1) / (2k+1)!
        float d = -1.0f / 93405312000.0f;
        d = fmaf(d, x, 1.0f / 518918400.0f);
        d = fmaf(d, x, -1.0f / 3991680.0f);
        d = fmaf(d, x, 1.0f / 45360.0f);
        d = fmaf(d, x, -1.0f / 840.0f);
        d = fmaf(d, x, 1.0f / 30.0f);
        d = fmaf(d, x, -1.0f / 3.0f);
        dS = a * d;
    } else {
        float sn, cs;
        sincos_mod(a, sn, cs);
        S = sn / a;
        C = cs;
        dS = (cs - S) / a;
    }
}

// Backward pass at one sample: recomputes the slow part with its derivatives
// and accumulates sum_c Y_c x'_c for x' in {x_P, x_C, dx/df0, dx/dfdot,
// dx/dfddot, dx/dlam, dx/dbeta} (7 complex accumulators in acc[14]).
//
// Reverse mode through the TDI combination: x_c = sum_q M_cq(omL) G_q with
// M in {0, +-fc2, +-fc2 fc} (gbgpu.py:370-375), so sum_c Y_c dx_c =
// sum_q Z_q dG_q + dOmL sum_q Zd_q G_q with the link adjoints
// Z_q = sum_c Y_c M_cq and Zd_q = sum_c Y_c dM_cq/domL.
//
// A link q (spacecraft s, arm a) is G = 1/4 sinc(a_q) e^{-i a_q} E_s A_a with
// a_q = fonfs_s hh_q, E_s = exp(-i phase_s), A_a = pp_a DP + cc_a DC.  Every
// parameter enters through fonfs_s, phase_s (per spacecraft), k.r_a, pp_a,
// cc_a (per arm) or omL, so the links are summed first into
//   U_s = sum_{q at s} hh_q (S'/S - i) Z_q G_q     (d/d fonfs_s)
//   V_s = -i sum_{q at s} Z_q G_q                   (d/d phase_s)
//   R_a = sum_{q on a} fonfs_s sg_q / 2 (S'/S - i) Z_q G_q   (d/d k.r_a)
//   Q_a = sum_{q on a} Z_q G_q / A_a               (d/d pp_a, cc_a: Q_a DP, Q_a DC)
//   W   = sum_q Zd_q G_q                            (d/d omL)
// and each parameter costs a few multiply-adds per spacecraft or arm.
//
// Third body (THIRD): fonfs carries the factor (1 + v_LOS/c) (vls: v_LOS of
// the three spacecraft at this sample), which scales its f0/fdot/fddot and
// k.P derivatives; the derivatives through v_LOS and the cumulative Doppler
// phase are left to the third-body pass, which takes cph[s] = V_s and
// cfo[s] = U_s.
template <bool THIRD>
__device__ __forceinline__ void slow_grad_mixed(const Bin &B, const GradExtra &Gx, int n, int N,
                                                dfl step, const double *__restrict__ tab,
                                                float ifs, float fstarf, const float2 Yc[3],
                                                const float2 Es[3], float acc[14],
                                                const float *vls = nullptr, float2 *cph = nullptr,
                                                float2 *cfo = nullptr)
{
    const float *tabf = reinterpret_cast<const float *>(tab + (size_t)18 * N);
    const float TWO_PI_F = (float)kTwoPi, PI_F = (float)kPi;
    // arm geometry: k.r, u.r, v.r, and the polarisation projections
    float kd[3], ru[3], rv[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float r0 = __ldg(tabf + (size_t)(3 * a) * N + n);
        float r1 = __ldg(tabf + (size_t)(3 * a + 1) * N + n);
        float r2 = __ldg(tabf + (size_t)(3 * a + 2) * N + n);
        kd[a] = fmaf(B.kf[0], r0, fmaf(B.kf[1], r1, B.kf[2] * r2));
        ru[a] = fmaf(Gx.u[0], r0, fmaf(Gx.u[1], r1, Gx.u[2] * r2));
        rv[a] = fmaf(Gx.v[0], r0, Gx.v[1] * r1);
    }
    // TDI factors and the link adjoints
    const dfl tm = df_mul_f(step, (float)n);
    const float tf = tm.h;
    const float omL = B.w0h + fmaf(fmaf(B.w2, tf, B.w1), tf, B.w0l);
    float so, co;
    sincos_mod(omL, so, co);
    const float2 fc = make_float2(co, -so);
    const float g4 = 4.0f * omL * so;
    const float2 fa = make_float2(g4 * co, -g4 * so);              // fc2
    const float2 fb = cmul(fa, fc);                                 // fc2 fc
    // d fc2 / d omL = 4 fc (sin + omL cos - i omL sin), d fc / d omL = -i fc
    const float2 da = cmul(make_float2(4.0f * fmaf(omL, co, so), -4.0f * omL * so), fc);
    const float2 db = cadd(cmul(da, fc), cmul(fa, make_float2(fc.y, -fc.x)));
    const float2 YA0 = cmul(Yc[0], fa), YA1 = cmul(Yc[1], fa), YA2 = cmul(Yc[2], fa);
    const float2 YB0 = cmul(Yc[0], fb), YB1 = cmul(Yc[1], fb), YB2 = cmul(Yc[2], fb);
    const float2 YdA0 = cmul(Yc[0], da), YdA1 = cmul(Yc[1], da), YdA2 = cmul(Yc[2], da);
    const float2 YdB0 = cmul(Yc[0], db), YdB1 = cmul(Yc[1], db), YdB2 = cmul(Yc[2], db);
    // spacecraft: delayed times and fonfs (FP32)
    float fo[3], xi[3], dop[3];
#pragma unroll
    for (int s = 0; s < 3; s++) {
        const float P0 = __ldg(tabf + (size_t)(9 + 3 * s) * N + n);
        const float P1 = __ldg(tabf + (size_t)(9 + 3 * s + 1) * N + n);
        const float P2 = __ldg(tabf + (size_t)(9 + 3 * s + 2) * N + n);
        const float kPf = fmaf(B.kf[0], P0, fmaf(B.kf[1], P1, B.kf[2] * P2));
        const float x = tf - kPf;
        xi[s] = x;
        const float f_ = B.w0h + fmaf(fmaf(B.w2, x, B.w1), x, B.w0l);
        dop[s] = THIRD ? 1.0f + vls[s] * (float)(1.0 / kCSI) : 1.0f;
        fo[s] = THIRD ? f_ * dop[s] : f_;
    }
    float2 A[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float pp = fmaf(rv[a], rv[a], -ru[a] * ru[a]);      // r.e+.r
        const float cc = 2.0f * ru[a] * rv[a];                       // r.ex.r
        A[a] = make_float2(fmaf(pp, B.DPf.x, cc * B.DCf.x), fmaf(pp, B.DPf.y, cc * B.DCf.y));
    }
    // links 12, 23, 31, 21, 32, 13: arm, spacecraft, sign of k.r
    const int arm[6] = {0, 1, 2, 0, 1, 2};
    const int sc[6] = {0, 1, 2, 1, 2, 0};
    const float sg[6] = {1.f, 1.f, 1.f, -1.f, -1.f, -1.f};
    float2 U[3], V[3], R[3], Q[3], W = {0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; k++) U[k] = V[k] = R[k] = Q[k] = make_float2(0.f, 0.f);
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const int s = sc[q], a = arm[q];
        // link adjoints (X = fa (G21 - G31) + fb (G12 - G13) and cyclic)
        float2 Z, Zd;
        switch (q) {
        case 0: Z = csub(YB0, YA1); Zd = csub(YdB0, YdA1); break;   // G12
        case 1: Z = csub(YB1, YA2); Zd = csub(YdB1, YdA2); break;   // G23
        case 2: Z = csub(YB2, YA0); Zd = csub(YdB2, YdA0); break;   // G31
        case 3: Z = csub(YA0, YB1); Zd = csub(YdA0, YdB1); break;   // G21
        case 4: Z = csub(YA1, YB2); Zd = csub(YdA1, YdB2); break;   // G32
        default: Z = csub(YA2, YB0); Zd = csub(YdA2, YdB0); break;  // G13
        }
        const float hh = 0.5f * fmaf(sg[q], kd[a], 1.0f);
        const float av = fo[s] * hh;
        float S, C, dS;
        sinc_cos_d_f(av, S, C, dS);
        const float t = 0.25f * S;
        const float2 gE = cmul(make_float2(t * C, -t * av * S), Es[s]);
        const float2 ZgE = cmul(Z, gE);
        const float2 ZG = cmul(ZgE, A[a]);
        const float2 G = cmul(gE, A[a]);
        W = cadd(W, cmul(Zd, G));
        Q[a] = cadd(Q[a], ZgE);
        const float dl = dS / S;
        const float2 w = make_float2(fmaf(dl, ZG.x, ZG.y), fmaf(dl, ZG.y, -ZG.x));   // (S'/S - i) Z G
        U[s] = make_float2(fmaf(hh, w.x, U[s].x), fmaf(hh, w.y, U[s].y));
        V[s] = make_float2(V[s].x + ZG.y, V[s].y - ZG.x);
        const float hf = 0.5f * sg[q] * fo[s];
        R[a] = make_float2(fmaf(hf, w.x, R[a].x), fmaf(hf, w.y, R[a].y));
    }
    // plus / cross parts: sum_a (pp_a, cc_a) Q_a
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float pp = fmaf(rv[a], rv[a], -ru[a] * ru[a]);
        const float cc = 2.0f * ru[a] * rv[a];
        acc[0] = fmaf(pp, Q[a].x, acc[0]);
        acc[1] = fmaf(pp, Q[a].y, acc[1]);
        acc[2] = fmaf(cc, Q[a].x, acc[2]);
        acc[3] = fmaf(cc, Q[a].y, acc[3]);
    }
    // frequency parameters: d fonfs_s = dop_s {1, xi, xi^2/2}/fstar, d phase_s =
    // -{2 pi xi, pi xi^2, pi/3 xi^3}, d omL = {1, tm, tm^2/2}/fstar
    {
        const float dom0 = ifs, dom1 = tf * ifs, dom2 = 0.5f * tf * tf * ifs;
        float2 s0 = {dom0 * W.x, dom0 * W.y}, s1 = {dom1 * W.x, dom1 * W.y},
               s2 = {dom2 * W.x, dom2 * W.y};
#pragma unroll
        for (int s = 0; s < 3; s++) {
            const float x = xi[s];
            const float c0 = dop[s] * ifs, c1 = c0 * x, c2 = 0.5f * c1 * x;
            const float p0 = -TWO_PI_F * x, p1 = -PI_F * x * x, p2 = -(PI_F / 3.0f) * x * x * x;
            s0 = make_float2(fmaf(c0, U[s].x, fmaf(p0, V[s].x, s0.x)), fmaf(c0, U[s].y, fmaf(p0, V[s].y, s0.y)));
            s1 = make_float2(fmaf(c1, U[s].x, fmaf(p1, V[s].x, s1.x)), fmaf(c1, U[s].y, fmaf(p1, V[s].y, s1.y)));
            s2 = make_float2(fmaf(c2, U[s].x, fmaf(p2, V[s].x, s2.x)), fmaf(c2, U[s].y, fmaf(p2, V[s].y, s2.y)));
        }
        acc[4] += s0.x; acc[5] += s0.y;
        acc[6] += s1.x; acc[7] += s1.y;
        acc[8] += s2.x; acc[9] += s2.y;
    }
    // sky angles: d/dlam (du = -ct v, dv = ct u - st k, dk = st v),
    //             d/dbeta (du = -k, dv = 0, dk = u);
    // per spacecraft d kP = (st v.P, u.P)/c moves phase_s by 2 pi f(xi) d kP
    // and fonfs_s by -(fdot + fddot xi)/fstar dop_s d kP
    {
        float2 sl = {0.f, 0.f}, sb = {0.f, 0.f};
#pragma unroll
        for (int s = 0; s < 3; s++) {
            const float P0 = __ldg(tabf + (size_t)(9 + 3 * s) * N + n);
            const float P1 = __ldg(tabf + (size_t)(9 + 3 * s + 1) * N + n);
            const float P2 = __ldg(tabf + (size_t)(9 + 3 * s + 2) * N + n);
            const float Pv = fmaf(Gx.v[0], P0, Gx.v[1] * P1);
            const float Pu = fmaf(Gx.u[0], P0, fmaf(Gx.u[1], P1, Gx.u[2] * P2));
            const float dkP_l = Gx.st * Pv, dkP_b = Pu;
            const float f_ = B.w0h + fmaf(fmaf(B.w2, xi[s], B.w1), xi[s], B.w0l);
            const float tpf = TWO_PI_F * f_ * fstarf;
            const float gfk = fmaf(Gx.gf1, xi[s], Gx.gf0) * dop[s];
            const float ul = gfk * dkP_l, ub = gfk * dkP_b;     // d fonfs_s
            const float vl_ = tpf * dkP_l, vb = tpf * dkP_b;    // d phase_s
            sl = make_float2(fmaf(ul, U[s].x, fmaf(vl_, V[s].x, sl.x)), fmaf(ul, U[s].y, fmaf(vl_, V[s].y, sl.y)));
            sb = make_float2(fmaf(ub, U[s].x, fmaf(vb, V[s].x, sb.x)), fmaf(ub, U[s].y, fmaf(vb, V[s].y, sb.y)));
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
            // d k.r_a, d pp_a, d cc_a per angle
            const float dkd_l = Gx.st * rv[a], dkd_b = ru[a];
            const float dru_l = -Gx.ct * rv[a], drv_l = fmaf(Gx.ct, ru[a], -Gx.st * kd[a]);
            const float dpp_l = 2.0f * fmaf(rv[a], drv_l, -ru[a] * dru_l);
            const float dcc_l = 2.0f * fmaf(dru_l, rv[a], ru[a] * drv_l);
            const float dpp_b = 2.0f * ru[a] * kd[a];
            const float dcc_b = -2.0f * kd[a] * rv[a];
            const float2 QP = cmul(Q[a], B.DPf), QC = cmul(Q[a], B.DCf);
            sl = make_float2(fmaf(dkd_l, R[a].x, fmaf(dpp_l, QP.x, fmaf(dcc_l, QC.x, sl.x))),
                             fmaf(dkd_l, R[a].y, fmaf(dpp_l, QP.y, fmaf(dcc_l, QC.y, sl.y))));
            sb = make_float2(fmaf(dkd_b, R[a].x, fmaf(dpp_b, QP.x, fmaf(dcc_b, QC.x, sb.x))),
                             fmaf(dkd_b, R[a].y, fmaf(dpp_b, QP.y, fmaf(dcc_b, QC.y, sb.y))));
        }
        acc[10] += sl.x; acc[11] += sl.y;
        acc[12] += sb.x; acc[13] += sb.y;
    }
    if (THIRD) {
#pragma unroll
        for (int s = 0; s < 3; s++) {
            cph[s] = V[s];
            cfo[s] = U[s];
        }
    }
}

// Adjoint of the third body's cumulative Doppler phase and of v_LOS at
// sample k (all three spacecraft).  With psi_n = (pi/c) sum_{m=1..n}
// dxi_m (g_{m-1} + g_m), g = v_LOS f_GW, dxi_m = xi_m - xi_{m-1}, and
// R_k = sum_{n>=k} cph_n (the suffix sums), the phase enters as -psi, so
//   sum_n cph_n d(-psi_n) = -(pi/c) sum_k [W_k dg_k + H_k dxi_k],
//   W_k = R_k dxi_k + R_{k+1} dxi_{k+1},  H_k = R_k (g_{k-1} + g_k) - R_{k+1} (g_k + g_{k+1})
// (terms outside 1 <= m <= N-1 dropped).  v_LOS also scales fonfs by
// (1 + v/c): sum cfo_k fo_base/c dv_k.  Accumulates into the f0, fdot,
// fddot, lam, beta slots (acc[4..13] of the 7-accumulator block) and the
// five third-body slots t5[10] (A2, varpi, e2, P2, T2).
__device__ __forceinline__ void third_grad_sample(const Bin &B, const GradExtra &Gx, int k, int N,
                                                  int lg, dfl stepd, const double *__restrict__ tab,
                                                  float ifs, const float2 *Rrow0, const float *grow0,
                                                  const float2 cfo[3], float acc[14], float t5[10])
{
    const float *tabf = reinterpret_cast<const float *>(tab + (size_t)18 * N);
    const float cpsi = -(float)(kPi / kCSI);
    const float ic = (float)(1.0 / kCSI);
    // as the forward pre-pass: one Kepler solve at spacecraft 1's delayed
    // time (float-pair time and mean anomaly, FP32 solve), the other
    // spacecraft linearised in their FP32 k.P/c offsets (<= 8.3 s: relative
    // change of dv[0..4] <= n2 8.3 s)
    const dfl xi0 = df_add(df_mul_f(stepd, (float)k), df_neg(kP1_pair(B, tabf, N, k)));
    float dv[6];
    const float v0 = vlos_grad_mixed(xi0, B, Gx.cosvarpi, Gx.P2yr, dv);
    const float x0 = xi0.h + xi0.l;
    const float sth = stepd.h, stl = stepd.l;
    auto kpf = [&](int s, int n) {
        const float *r = tabf + (size_t)(9 + 3 * s) * N + n;
        return fmaf(B.kf[0], __ldg(r), fmaf(B.kf[1], __ldg(r + N), B.kf[2] * __ldg(r + 2 * N)));
    };
    const float kPf0 = kpf(0, k);
#pragma unroll
    for (int s = 0; s < 3; s++) {
        const float2 *Rrow = Rrow0 + (size_t)s * N;
        const float *grow = grow0 + (size_t)s * N;
        const float kPk = s ? kpf(s, k) : kPf0;
        const float dk = kPk - kPf0;
        const float v = fmaf(-dv[5], dk, v0);
        const float xf = x0 - dk;
        const float fgw = fmaf(fmaf(0.5f * B.fddotf, xf, B.fdotf), xf, B.f0f);
        const float fgwd = fmaf(B.fddotf, xf, B.fdotf);
        const float gk = grow[k];
        float2 W = {0.f, 0.f}, H = {0.f, 0.f};
        if (k >= 1) {
            const float dxi = (sth - (kPk - kpf(s, k - 1))) + stl;     // xi_k - xi_{k-1}
            const float2 R = Rrow[swz(k, lg)];
            const float gs = grow[k - 1] + gk;
            W = make_float2(R.x * dxi, R.y * dxi);
            H = make_float2(R.x * gs, R.y * gs);
        }
        if (k <= N - 2) {
            const float dxi = (sth - (kpf(s, k + 1) - kPk)) + stl;     // xi_{k+1} - xi_k
            const float2 R = Rrow[swz(k + 1, lg)];
            const float gs = gk + grow[k + 1];
            W = make_float2(fmaf(R.x, dxi, W.x), fmaf(R.y, dxi, W.y));
            H = make_float2(fmaf(-R.x, gs, H.x), fmaf(-R.y, gs, H.y));
        }
        // f0, fdot, fddot: dg = v {1, xi, xi^2/2}
        const float wv = cpsi * v;
        const float w1 = wv * xf, w2 = 0.5f * wv * xf * xf;
        acc[4] = fmaf(wv, W.x, acc[4]);
        acc[5] = fmaf(wv, W.y, acc[5]);
        acc[6] = fmaf(w1, W.x, acc[6]);
        acc[7] = fmaf(w1, W.y, acc[7]);
        acc[8] = fmaf(w2, W.x, acc[8]);
        acc[9] = fmaf(w2, W.y, acc[9]);
        // sky angles: dxi = -dkP, dg = g' dxi, dv = v' dxi
        const float cv = fgw * ifs * ic;                 // d fonfs / d v = fo_base / c
        const float gd = fmaf(dv[5], fgw, v * fgwd);
        const float q5 = cv * dv[5];
        const float2 Q = make_float2(-cpsi * fmaf(W.x, gd, H.x) - q5 * cfo[s].x,
                                     -cpsi * fmaf(W.y, gd, H.y) - q5 * cfo[s].y);
        const float P0 = __ldg(tabf + (size_t)(9 + 3 * s) * N + k);
        const float P1 = __ldg(tabf + (size_t)(9 + 3 * s + 1) * N + k);
        const float P2 = __ldg(tabf + (size_t)(9 + 3 * s + 2) * N + k);
        const float dkP_l = Gx.st * fmaf(Gx.v[0], P0, Gx.v[1] * P1);
        const float dkP_b = fmaf(Gx.u[0], P0, fmaf(Gx.u[1], P1, Gx.u[2] * P2));
        acc[10] = fmaf(Q.x, dkP_l, acc[10]);
        acc[11] = fmaf(Q.y, dkP_l, acc[11]);
        acc[12] = fmaf(Q.x, dkP_b, acc[12]);
        acc[13] = fmaf(Q.y, dkP_b, acc[13]);
        // third-body parameters: dg = f_GW dv, d fonfs = fo_base/c dv
        const float wf = cpsi * fgw;
        const float2 Tc = make_float2(fmaf(wf, W.x, cv * cfo[s].x), fmaf(wf, W.y, cv * cfo[s].y));
#pragma unroll
        for (int j = 0; j < 5; j++) {
            t5[2 * j] = fmaf(Tc.x, dv[j], t5[2 * j]);
            t5[2 * j + 1] = fmaf(Tc.y, dv[j], t5[2 * j + 1]);
        }
    }
}

// In-place decimation-in-time FFT on bit-reversed input (natural-order output)
// over `nsub` sub-arrays of length N = 2^lg: the five smallest half-spans
// inside warps with shuffles, the rest in register passes of up to three
// stages (the mirror image of fft_dif).
template <typename R, int RB>
__device__ __forceinline__ void fft_dit_pass(typename C2<R>::T *buf, int nsub, int lg, int hl)
{
    using V = typename C2<R>::T;
    constexpr int M = 1 << RB;
    const int groups = nsub << (lg - RB);
    for (int g = threadIdx.x; g < groups; g += kBlock) {
        const int a = g >> (lg - RB);
        const int rem = g & ((1 << (lg - RB)) - 1);
        const int blk = rem >> hl;
        const int r = rem & ((1 << hl) - 1);
        V *sub = buf + ((size_t)a << lg);
        const int p0 = (blk << (hl + RB)) + r;
        V x[M];
#pragma unroll
        for (int m = 0; m < M; m++) x[m] = sub[swz(p0 + (m << hl), lg)];
#pragma unroll
        for (int j = 0; j < RB; j++) {
            const int dm = 1 << j;
            const int hh = hl + j;
            const int ts = kTwN >> (hh + 1);
#pragma unroll
            for (int m = 0; m < M; m++) {
                if (m & dm) continue;
                const int rp = r + ((m & (dm - 1)) << hl);
                V t = cmul(tw<R>(rp * ts), x[m + dm]);
                V u = x[m];
                x[m] = cadd(u, t);
                x[m + dm] = csub(u, t);
            }
        }
#pragma unroll
        for (int m = 0; m < M; m++) sub[swz(p0 + (m << hl), lg)] = x[m];
    }
}

template <typename R>
__device__ __forceinline__ void fft_dit(typename C2<R>::T *buf, int nsub, int lg)
{
    using V = typename C2<R>::T;
    // the first five stages inside a warp: (a, b) -> (a + W b, a - W b) with a
    // on the lower lane; the upper lane multiplies its own element by W
    // before the exchange (w' = 1 on lower lanes and in the first stage), so
    // both lanes finish with sg x' + y' (sg = +-1): branch-free
    const int lane = threadIdx.x & 31;
    V w[5];
    R sg[5];
#pragma unroll
    for (int k = 0; k < 5; k++) {
        const bool up = (lane & (1 << k)) != 0;
        const int rp = lane & ((1 << k) - 1);
        sg[k] = up ? (R)-1 : (R)1;
        w[k] = up ? tw<R>(rp * (kTwN >> (k + 1))) : V{(R)1, (R)0};
    }
    const int chunks = (nsub << lg) >> 5;
    for (int c = threadIdx.x >> 5; c < chunks; c += kBlock >> 5) {
        const int e = (c << 5) + lane;
        const int idx = ((e >> lg) << lg) + swz(e & ((1 << lg) - 1), lg);
        V x = buf[idx];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const V xw = (k > 0) ? cmul(w[k], x) : x;
            const V y = shfl_c<R>(xw, 1 << k);
            x = V{fma(sg[k], xw.x, y.x), fma(sg[k], xw.y, y.y)};
        }
        buf[idx] = x;
    }
    __syncthreads();
    int hl = 5;
    while (hl < lg) {
        const int rb = (lg - hl) >= 3 ? 3 : (lg - hl);
        if (rb == 3) fft_dit_pass<R, 3>(buf, nsub, lg, hl);
        else if (rb == 2) fft_dit_pass<R, 2>(buf, nsub, lg, hl);
        else fft_dit_pass<R, 1>(buf, nsub, lg, hl);
        hl += rb;
        __syncthreads();
    }
}

struct GradParams {
    KParams K;
    double *grad;                  // (nparams, num_bin) FP64, the params layout
};

// accumulators per thread: ll terms 3, Qf 2, 7 complex (P, C, f0, fdot, fddot,
// lam, beta) 14; the third body adds 5 complex (A2, varpi, e2, P2, T2)
template <bool THIRD> __host__ __device__ constexpr int grad_acc() { return THIRD ? 29 : 19; }

// shared memory of a grad_kernel tile of maxS samples
// (buf: A and E per sample, 2 float2; es: 3 float2; third body: psi 3
// doubles, v_LOS and g 3 floats each)
__host__ __device__ constexpr size_t grad_smem_bytes(bool third, int maxS, int maxP)
{
    return (sizeof(Bin) + sizeof(GradExtra)) * (size_t)maxP + sizeof(double) * (third ? 29 : 19) * 2 * kMaxPack +
           (size_t)maxS * (5 * sizeof(float2) + (third ? 3 * (sizeof(double) + 2 * sizeof(float)) : 0));
}

// SWAP: binaries 2j (the current source, h_o) and 2j+1 (the proposal, h) of
// each tile form a pair, both transformed in the forward pass; only the
// proposal is differentiated, against the data r + h_o (r: the residual row),
// since d/dtheta [Re<r|h - h_o> - 1/2 <h - h_o|h - h_o>] = Re<r + h_o - h|dh>.
// Its gradient goes to column j of grad (num_bin / 2 columns), and d_h, h_h
// (when given) receive <r + h_o|h> and <h|h>.
template <bool THIRD, bool SWAP>
__global__ void __launch_bounds__(kBlock, 2) grad_kernel(const GradParams GP)
{
    using V = float2;
    constexpr int kGradAcc = grad_acc<THIRD>();
    const float is2 = 0.70710678118654752440f, is6 = 0.40824829046386301637f;
    const KParams &K = GP.K;
    extern __shared__ __align__(16) unsigned char smem[];
    Bin *bins = reinterpret_cast<Bin *>(smem);
    GradExtra *gxs = reinterpret_cast<GradExtra *>(smem + sizeof(Bin) * K.maxP);
    double *red = reinterpret_cast<double *>(smem + (sizeof(Bin) + sizeof(GradExtra)) * K.maxP);
    // red: group partial sums (float pairs, up to kMaxPack groups) and
    // per-binary FP64 sums (up to kMaxPack binaries), kMaxPack x kGradAcc each
    V *buf = reinterpret_cast<V *>(smem + (sizeof(Bin) + sizeof(GradExtra)) * K.maxP +
                                   sizeof(double) * kGradAcc * 2 * kMaxPack);
    // buf: the A and E channels (forward transform, then the adjoint's);
    // es: exp(-i phase_s) per sample from the forward pass, directly after buf
    // (the third-body pre-passes use buf and es together as FP64 scratch)
    V *es = buf + 2 * (size_t)K.maxS;
    // third body: cumulative phase as float pairs (forward; reused for the
    // phase adjoints cph in the backward pass), v_LOS and g = v_LOS f_GW per
    // (sample, spacecraft)
    dfl *psi = reinterpret_cast<dfl *>(es + 3 * (size_t)K.maxS);
    float2 *cphs = reinterpret_cast<float2 *>(psi);
    float *vl = reinterpret_cast<float *>(psi + 3 * (size_t)K.maxS);
    float *gq = vl + 3 * (size_t)K.maxS;
    __shared__ int s_tile;

    const gbx_wave_args &a = K.a;
    const int tid = threadIdx.x;
    const int ntiles = a.tiles ? a.ntiles : (a.num_bin + K.P - 1) / K.P;
    const float ifs = (float)(1.0 / K.fstar);
    const float fstarf = (float)K.fstar;
    const float Loc = (float)(1.0 / (kTwoPi * K.fstar));    // L / c
    const Bin *wsb = static_cast<const Bin *>(a.workspace);
    const GradExtra *wsg = reinterpret_cast<const GradExtra *>(wsb + a.num_bin);
    int iter = 0;
    for (;;) {
        if (tid == 0) s_tile = a.queue ? atomicAdd(a.queue, 1) : (int)(blockIdx.x + iter * gridDim.x);
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
        const int maxcnt = tile_pack(a.tile, lg, SWAP ? 2 : 1);
        if (tab == nullptr || cnt < 1 || cnt > maxcnt || first < 0 || first + cnt > a.num_bin ||
            (cnt << lg) > K.maxS || (SWAP && ((cnt | first) & 1))) {
            flag(a.status, GBX_FLAG_TILE);
            __syncthreads();
            continue;
        }
        {
            const int4 *src = reinterpret_cast<const int4 *>(wsb + first);
            int4 *dst = reinterpret_cast<int4 *>(bins);
            for (int k = tid; k < cnt * (int)(sizeof(Bin) / 16); k += kBlock) dst[k] = src[k];
            const int4 *src2 = reinterpret_cast<const int4 *>(wsg + first);
            int4 *dst2 = reinterpret_cast<int4 *>(gxs);
            for (int k = tid; k < cnt * (int)(sizeof(GradExtra) / 16); k += kBlock) dst2[k] = src2[k];
        }
        __syncthreads();
        const int S = cnt << lg;
        const dfl stepd = K.stepd[lg];
        // (scratch for the pre-pass: k.P/c of every sample in buf)
        if (THIRD) third_prepass_mixed(bins, tab, cnt, lg, stepd, psi, vl, reinterpret_cast<float *>(buf), gq);

        // forward slow part and FFT
        for (int m = tid; m < S; m += kBlock) {
            const int p = m >> lg, n = m & (N - 1);
            float2 o[3];
            dfl ps[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
            float vv[3] = {0.f, 0.f, 0.f};
            if (THIRD) {
#pragma unroll
                for (int s = 0; s < 3; s++) {
                    ps[s] = psi[(p * 3 + s) * N + n];
                    vv[s] = vl[(p * 3 + s) * N + n];
                }
            }
            slow_mixed<THIRD, true>(bins[p], n, N, stepd, Loc, tab, ps, vv, o, es + 3 * (size_t)m);
            // A and E before the (linear) transform
            buf[(p * 2 + 0) * N + swz(n, lg)] = {(o[2].x - o[0].x) * is2, (o[2].y - o[0].y) * is2};
            buf[(p * 2 + 1) * N + swz(n, lg)] = {(o[0].x - 2.f * o[1].x + o[2].x) * is6,
                                                 (o[0].y - 2.f * o[1].y + o[2].y) * is6};
        }
        __syncthreads();
        fft_dif<float>(buf, 2 * cnt, lg);

        // residual weights, likelihood terms, Qf; conj(w) written in place.
        // Tpb threads per differentiated binary p (with SWAP, the odd ones)
        const int Tpb = (SWAP ? 2 : 1) * (kBlock / maxcnt);
        const int width = Tpb < 32 ? Tpb : 32;
        const int pq = tid / Tpb;
        const int p = SWAP ? 2 * pq + 1 : pq;
        const int i0 = tid - pq * Tpb;
        const int nproc = SWAP ? cnt >> 1 : cnt;
        const bool valid = p < cnt && bins[p].valid && (!SWAP || bins[p - 1].valid);
        float acc[kGradAcc];
#pragma unroll
        for (int k = 0; k < kGradAcc; k++) acc[k] = 0.0f;
        if (p < cnt) {
            const Bin &B = bins[p];
            bool out = false;
            // scale 2^eD as a float complex: h in the data's scaled units
            const float2 sc = make_float2(d2f_scaled(B.scale.x, B.eD), d2f_scaled(B.scale.y, B.eD));
            // SWAP: the current source's scale in the same units
            const Bin &Bo = bins[SWAP ? p - 1 : p];
            const float2 so = make_float2(d2f_scaled(Bo.scale.x, B.eD), d2f_scaled(Bo.scale.y, B.eD));
            for (int i = i0; i < N; i += Tpb) {
                const int j = B.start + i;
                const int pos = bitrev((i + (N >> 1)) & (N - 1), lg);
                const int sp = swz(pos, lg);
                const V hA = buf[(p * 2 + 0) * N + sp], hE = buf[(p * 2 + 1) * N + sp];
                float2 uA = {0.f, 0.f}, uE = {0.f, 0.f};
                if (valid && j >= 0 && j < K.L) {
                    const size_t jd = (size_t)B.di * K.L + j, jn = (size_t)B.ni * K.L + j;
                    const double2 dA = __ldg(K.A_data + jd), dE = __ldg(K.E_data + jd);
                    // one PSD array for both channels: one weight, and the
                    // likelihood terms summed as the fused likelihood sums them
                    const bool samepsd = K.A_psd == K.E_psd;
                    const double SA = __ldg(K.A_psd + jn);
                    const float wA = __frcp_rn(d2f_scaled(SA, B.eS));
                    const float wE = samepsd ? wA : __frcp_rn(d2f_scaled(__ldg(K.E_psd + jn), B.eS));
                    float aR = d2f_scaled(dA.x, B.eD), aI = d2f_scaled(dA.y, B.eD);
                    float eR = d2f_scaled(dE.x, B.eD), eI = d2f_scaled(dE.y, B.eD);
                    if (SWAP) {
                        // data r + h_o: the current source on the windows' overlap
                        const int k = j - Bo.start;
                        if (k >= 0 && k < N) {
                            const int pk = swz(bitrev((k + (N >> 1)) & (N - 1), lg), lg);
                            const float2 oA = cmul(so, buf[((p - 1) * 2 + 0) * N + pk]);
                            const float2 oE = cmul(so, buf[((p - 1) * 2 + 1) * N + pk]);
                            aR += oA.x; aI += oA.y;
                            eR += oE.x; eI += oE.y;
                        }
                    }
                    if (samepsd) {
                        acc[0] = fmaf(fmaf(aR, hA.x, aI * hA.y) + fmaf(eR, hE.x, eI * hE.y), wA, acc[0]);
                        acc[1] = fmaf(fmaf(aR, hA.y, -aI * hA.x) + fmaf(eR, hE.y, -eI * hE.x), wA, acc[1]);
                        acc[2] = fmaf(fmaf(hA.x, hA.x, hA.y * hA.y) + fmaf(hE.x, hE.x, hE.y * hE.y), wA, acc[2]);
                    } else {
                        acc[0] += fmaf(aR, hA.x, aI * hA.y) * wA + fmaf(eR, hE.x, eI * hE.y) * wE;
                        acc[1] += fmaf(aR, hA.y, -aI * hA.x) * wA + fmaf(eR, hE.y, -eI * hE.x) * wE;
                        acc[2] += fmaf(hA.x, hA.x, hA.y * hA.y) * wA + fmaf(hE.x, hE.x, hE.y * hE.y) * wE;
                    }
                    // r' = d' - sc h ; u = r' / S'
                    const float2 shA = cmul(sc, hA), shE = cmul(sc, hE);
                    uA = make_float2((aR - shA.x) * wA, (aI - shA.y) * wA);
                    uE = make_float2((eR - shE.x) * wE, (eI - shE.y) * wE);
                    // Qf = sum_c conj(w_c) x_c = conj(uA) hA + conj(uE) hE (the
                    // X, Y, Z weights are the A, E ones mapped back)
                    acc[3] += fmaf(uA.x, hA.x, fmaf(uA.y, hA.y, fmaf(uE.x, hE.x, uE.y * hE.y)));
                    acc[4] += fmaf(uA.x, hA.y, fmaf(-uA.y, hA.x, fmaf(uE.x, hE.y, -uE.y * hE.x)));
                } else if (valid) {
                    out = true;
                }
                buf[(p * 2 + 0) * N + sp] = make_float2(uA.x, -uA.y);
                buf[(p * 2 + 1) * N + sp] = make_float2(uE.x, -uE.y);
            }
            if (out) flag(a.status, GBX_FLAG_WINDOW);
        }
        __syncthreads();
        fft_dit<float>(buf, 2 * cnt, lg);

        // backward pass: Y_c,n at natural position n
        if (p < cnt) {
            const Bin &B = bins[p];
            const GradExtra &Gx = gxs[p];
            if (valid) {
                for (int n = i0; n < N; n += Tpb) {
                    float2 Yc[3], Es[3];
                    float2 *ep = es + 3 * ((size_t)(p << lg) + n);
                    // Y_X, Y_Y, Y_Z from the transformed A, E weights
                    const V YA = buf[(p * 2 + 0) * N + swz(n, lg)], YE = buf[(p * 2 + 1) * N + swz(n, lg)];
                    Yc[0] = make_float2(fmaf(-YA.x, is2, YE.x * is6), fmaf(-YA.y, is2, YE.y * is6));
                    Yc[1] = make_float2(-2.f * YE.x * is6, -2.f * YE.y * is6);
                    Yc[2] = make_float2(fmaf(YA.x, is2, YE.x * is6), fmaf(YA.y, is2, YE.y * is6));
#pragma unroll
                    for (int c = 0; c < 3; c++) Es[c] = ep[c];
                    if (THIRD) {
                        // cph goes to the (now free) psi rows, cfo replaces exp(-i phase)
                        // in this thread's own slots
                        float vv[3];
                        float2 cph[3], cfo[3];
#pragma unroll
                        for (int s = 0; s < 3; s++) vv[s] = vl[(p * 3 + s) * N + n];
                        slow_grad_mixed<true>(B, Gx, n, N, stepd, tab, ifs, fstarf, Yc, Es, acc + 5,
                                              vv, cph, cfo);
#pragma unroll
                        for (int s = 0; s < 3; s++) {
                            cphs[(p * 3 + s) * N + swz(n, lg)] = cph[s];
                            ep[s] = cfo[s];
                        }
                    } else {
                        slow_grad_mixed<false>(B, Gx, n, N, stepd, tab, ifs, fstarf, Yc, Es, acc + 5);
                    }
                }
            }
        }
        if (THIRD) {
            __syncthreads();
            // suffix sums R_k = sum_{n >= k} cph_n along every (binary, spacecraft) row
            const int warp = tid >> 5, lane = tid & 31;
            const int chunk = N >> 5;
            for (int rr = warp; rr < 3 * nproc; rr += kBlock / 32) {
                const int row = SWAP ? 3 * (2 * (rr / 3) + 1) + rr % 3 : rr;
                V *rp = cphs + (size_t)row * N;
                const int c0 = lane * chunk;
                float2 t = {0.f, 0.f};
                for (int c = 0; c < chunk; c++) t = cadd(t, rp[swz(c0 + c, lg)]);
                float2 incl = t;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    float2 y = make_float2(__shfl_down_sync(0xffffffffu, incl.x, o),
                                           __shfl_down_sync(0xffffffffu, incl.y, o));
                    if (lane + o < 32) incl = cadd(incl, y);
                }
                float2 run = csub(incl, t);
                for (int c = chunk - 1; c >= 0; c--) {
                    run = cadd(run, rp[swz(c0 + c, lg)]);
                    rp[swz(c0 + c, lg)] = run;
                }
            }
            __syncthreads();
            if (valid) {
                const Bin &B = bins[p];
                const GradExtra &Gx = gxs[p];
                for (int k = i0; k < N; k += Tpb) {
                    const float2 *cf = es + 3 * ((size_t)(p << lg) + k);
                    const float2 cfo[3] = {cf[0], cf[1], cf[2]};
                    third_grad_sample(B, Gx, k, N, lg, stepd, tab, ifs, cphs + (size_t)(p * 3) * N,
                                      gq + (size_t)(p * 3) * N, cfo, acc + 5, acc + 19);
                }
            }
        }
        // Reduction: float-pair trees within groups of `width` lanes; group
        // leaders store the pairs; then one thread per (binary, accumulator)
        // adds its groups and converts to FP64 once, and one thread per
        // (binary, output) forms the result.  Spreading the FP64 work over
        // lanes keeps it off the critical path (the FP64 pipe issues a warp
        // instruction per 64 cycles per SM sub-partition, whatever the mask).
        float2 *red2 = reinterpret_cast<float2 *>(red);
        double *tsum = red + kGradAcc * kMaxPack;
        {
            const bool leader = (tid & (width - 1)) == 0;
            const int g = tid / width;
#pragma unroll
            for (int k = 0; k < kGradAcc; k++) {
                dfl x = {acc[k], 0.f};
                for (int o = width >> 1; o > 0; o >>= 1) {
                    dfl y = {__shfl_xor_sync(0xffffffffu, x.h, o), __shfl_xor_sync(0xffffffffu, x.l, o)};
                    x = df_add(x, y);
                }
                if (leader) red2[kGradAcc * g + k] = make_float2(x.h, x.l);
            }
        }
        __syncthreads();
        {
            const int per = Tpb / width;
            for (int t = tid; t < nproc * kGradAcc; t += kBlock) {
                const int q = t / kGradAcc, k = t - q * kGradAcc;
                dfl x = {0.f, 0.f};
                for (int g = q * per; g < (q + 1) * per; g++) {
                    const float2 y = red2[kGradAcc * g + k];
                    x = df_add(x, dfl{y.x, y.y});
                }
                tsum[t] = (double)x.h + (double)x.l;
            }
        }
        __syncthreads();
        {
            constexpr int kOut = (THIRD ? 14 : 9) + 1;   // gradient rows + (d_h, h_h)
            for (int t = tid; t < nproc * kOut; t += kBlock) {
                const int q = t / kOut, j = t - q * kOut;
                const int bq = SWAP ? 2 * q + 1 : q;
                const Bin &B = bins[bq];
                if (B.b < 0) continue;
                const bool ok = B.valid && (!SWAP || (bins[bq - 1].valid && bins[bq - 1].b >= 0));
                const int col = SWAP ? B.b >> 1 : B.b;
                const GradExtra &Gx = gxs[bq];
                const double *ts = tsum + q * kGradAcc;
                const double s4 = 4.0 * K.df;
                // weights were 4 df r / S in units of 2^(eS - eD): cu converts sums of w
                const double cu = s4 * exp2_int(B.eS - B.eD);
                const double2 sc = B.scale;
                const size_t nb = SWAP ? a.num_bin >> 1 : a.num_bin;
                if (j == kOut - 1) {
                    const double ch = s4 * exp2_int(B.eS) * (sc.x * sc.x + sc.y * sc.y);
                    const double2 dh = cmul(make_double2(cu * ts[0], cu * ts[1]), sc);
                    if (K.d_h) K.d_h[col] = ok ? dh : make_double2(0.0, 0.0);
                    if (K.h_h) K.h_h[col] = ok ? make_double2(ch * ts[2], 0.0) : make_double2(0.0, 0.0);
                    continue;
                }
                double g;
                if (j == 0 || j == 1 || j == 4) {
                    const double2 scQf = cmul(sc, make_double2(cu * ts[3], cu * ts[4]));
                    if (j == 0) g = scQf.x / a.params[B.b];                       // amp
                    else if (j == 4) g = -scQf.y;                                  // phi0: Re(i sc Qf)
                    else g = cmul(sc, make_double2(cu * ts[9], cu * ts[10])).x +   // f0
                             cmul(Gx.dlnsc_f0, scQf).x;
                } else if (j == 5 || j == 6) {                                     // iota, psi
                    const double2 QP = make_double2(cu * ts[5], cu * ts[6]);
                    const double2 QC = make_double2(cu * ts[7], cu * ts[8]);
                    const double2 dP = j == 5 ? Gx.dDPi : Gx.dDPp, dC = j == 5 ? Gx.dDCi : Gx.dDCp;
                    g = cmul(sc, cadd(cmul(dP, QP), cmul(dC, QC))).x;
                } else {
                    // fdot 11, fddot 13, lam 15, beta 17; third body 19 + 2 (j - 9)
                    const int k = j == 2 ? 11 : j == 3 ? 13 : j == 7 ? 15 : j == 8 ? 17 : 19 + 2 * (j - 9);
                    g = cmul(sc, make_double2(cu * ts[k], cu * ts[k + 1])).x;
                }
                GP.grad[(size_t)j * nb + col] = ok ? g : 0.0;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kPrepBlock) prep_grad_kernel(const KParams K)
{
    extern __shared__ __align__(16) unsigned char smem[];
    Bin *sb = reinterpret_cast<Bin *>(smem);
    GradExtra *sg = reinterpret_cast<GradExtra *>(smem + sizeof(Bin) * kPrepBlock);
    const gbx_wave_args &a = K.a;
    const int s0 = blockIdx.x * kPrepBlock;
    const int slot = s0 + threadIdx.x;
    if (slot < a.num_bin) {
        int lg;
        if (a.tiles) {
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
            memset(&sg[threadIdx.x], 0, sizeof(GradExtra));
            sb[threadIdx.x].b = -1;
        } else {
            setup_bin(sb[threadIdx.x], K, b, 1 << lg, MODE_LL);
            setup_grad(sg[threadIdx.x], K, b);
        }
    }
    __syncthreads();
    const int cnt = min(kPrepBlock, a.num_bin - s0);
    Bin *wsb = static_cast<Bin *>(a.workspace);
    GradExtra *wsg = reinterpret_cast<GradExtra *>(wsb + a.num_bin);
    const int4 *src = reinterpret_cast<const int4 *>(sb);
    int4 *dst = reinterpret_cast<int4 *>(wsb + s0);
    for (int k = threadIdx.x; k < cnt * (int)(sizeof(Bin) / 16); k += kPrepBlock) dst[k] = src[k];
    const int4 *src2 = reinterpret_cast<const int4 *>(sg);
    int4 *dst2 = reinterpret_cast<int4 *>(wsg + s0);
    for (int k = threadIdx.x; k < cnt * (int)(sizeof(GradExtra) / 16); k += kPrepBlock)
        dst2[k] = src2[k];
}
