// Per-binary Fisher matrices F_ij = <dh/dtheta_i | dh/dtheta_j> of the nine
// parameters (amp, f0, fdot, fddot, phi0, iota, psi, lam, beta) by forward
// mode, in one launch: the reference forms them from five-point differences
// of run_wave, 4 launches per parameter (gbgpu/gbgpu.py:957-1138), with the
// inner product 4 df sum_{A,E} Re conj(a) b / S of its likelihood.
//
// h = scale FFT(x) with x = DP x^P + DC x^C (the slow part is linear in the
// polarisation amplitudes DP, DC), so per sample the kernel forms seven rows
// of the A and E channels: the bases x^P, x^C and the tangents dx/dtheta for
// theta = f0 T, fdot T^2, fddot T^3, lam, beta (frequency parameters in units
// of 1/T^k so that every row is O(1) in FP32).  After the 14 transforms:
//   dh/d amp = h/amp,  dh/d phi0 = i h,
//   dh/d iota = scale (dDP/diota X^P + dDC/diota X^C), psi alike,
//   dh/d f0 = scale (dX/d(f0 T) + d ln scale/d(f0 T) X) / T,
// and the rest are the transformed tangents; the 45 products of the upper
// triangle are summed per bin in FP32, over lanes and groups in float pairs,
// and scaled back to the parameters' units in FP64.
//
// Tangents follow the derivative structure of the gradient kernel's slow
// part (gbx_grad.cuh): a link G_q = 1/4 sinc(a_q) e^{-i a_q} E_s A_a moves by
//   dG_q = G_q [(S'/S - i) d a_q - i d phase_s] + gE_q dA_a,
//   d a_q = hh_q d fonfs_s + fonfs_s sg_q / 2 d k.r_a,
// and X = fa (G21 - G31) + fb (G12 - G13) (Y, Z cyclic) adds d omL (da, db).
//
// This file is included inside namespace gbx by gbx_wave.cu.

constexpr int kFisherRows = 7;           // x^P, x^C, f0 T, fdot T^2, fddot T^3, lam, beta
constexpr int kFisherPar = 9;
constexpr int kFisherAcc = kFisherPar * (kFisherPar + 1) / 2;

__host__ __device__ constexpr size_t fisher_smem_bytes(int maxS, int maxP)
{
    return (sizeof(Bin) + sizeof(GradExtra)) * (size_t)maxP + sizeof(double) * kFisherAcc * 2 * kMaxPack +
           (size_t)maxS * 2 * kFisherRows * sizeof(float2);
}

// The seven rows at sample n; outA[r], outE[r] are the A and E channels.
__device__ __forceinline__ void slow_tangent_mixed(const Bin &B, const GradExtra &Gx, int n, int N,
                                                   dfl step, float Loc,
                                                   const double *__restrict__ tab, float ifs,
                                                   float fstarf, float iT, float2 outA[kFisherRows],
                                                   float2 outE[kFisherRows])
{
    const float *tabf = reinterpret_cast<const float *>(tab + (size_t)18 * N);
    const float TWO_PI_F = (float)kTwoPi, PI_F = (float)kPi;
    const float is2 = 0.70710678118654752440f, is6 = 0.40824829046386301637f;
    float kd[3], ru[3], rv[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float r0 = __ldg(tabf + (size_t)(3 * a) * N + n);
        const float r1 = __ldg(tabf + (size_t)(3 * a + 1) * N + n);
        const float r2 = __ldg(tabf + (size_t)(3 * a + 2) * N + n);
        kd[a] = fmaf(B.kf[0], r0, fmaf(B.kf[1], r1, B.kf[2] * r2));
        ru[a] = fmaf(B.uf[0], r0, fmaf(B.uf[1], r1, B.uf[2] * r2));
        rv[a] = fmaf(B.vf[0], r0, B.vf[1] * r1);
    }
    // carrier phases exactly as slow_mixed (circular model)
    const dfl twopi = df_from(kTwoPi);
    const dfl tm = df_mul_f(step, (float)n);
    const float tf = tm.h;
    dfl Phi0 = df_add(df_mul(B.omdfad, tm), B.phi0d);
    const dfl tm2 = df_mul(tm, tm);
    Phi0 = df_add(Phi0, df_mul(tm2, df_fast(B.pfd.h, fmaf(B.p3d.h, tf, B.pfd.l))));
    Phi0 = df_neg(Phi0);
    const dfl wt = df_add(B.omd, df_add(df_mul(B.tpfd, tm), dfl{B.pfddd.h * tf * tf, 0.0f}));
    const float fdt = fmaf(B.fddotf, tf, B.fdotf);
    const dfl kP0 = kP1_pair(B, tabf, N, n);
    dfl ph0 = df_add(Phi0, df_mul(kP0, wt));
    {
        const float q = rintf(ph0.h * (float)kInvTwoPi);
        ph0 = df_add(ph0, df_neg(df_mul_f(twopi, q)));
    }
    const float dk[3] = {0.0f, Loc * kd[0], -Loc * kd[2]};
    float2 Es[3];
    float fo[3], xs[3], tau[3], dkPl[3], dkPb[3];
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
        float sn, cs;
        sincos_mod(ph.h, sn, cs);
        Es[s] = make_float2(fmaf(sn, -ph.l, cs), -fmaf(cs, ph.l, sn));
        const float xf = tf - kPf;
        fo[s] = B.w0h + fmaf(fmaf(B.w2, xf, B.w1), xf, B.w0l);
        xs[s] = xf;
        tau[s] = xf * iT;
        const float P0 = __ldg(tabf + (size_t)(9 + 3 * s) * N + n);
        const float P1 = __ldg(tabf + (size_t)(9 + 3 * s + 1) * N + n);
        const float P2 = __ldg(tabf + (size_t)(9 + 3 * s + 2) * N + n);
        dkPl[s] = Gx.st * fmaf(Gx.v[0], P0, Gx.v[1] * P1);
        dkPb[s] = fmaf(Gx.u[0], P0, fmaf(Gx.u[1], P1, Gx.u[2] * P2));
    }
    // TDI factors fa = fc2, fb = fc2 fc and their omL derivatives
    const float omL = B.w0h + fmaf(fmaf(B.w2, tf, B.w1), tf, B.w0l);
    float so, co;
    sincos_mod(omL, so, co);
    const float2 fc = make_float2(co, -so);
    const float g4 = 4.0f * omL * so;
    const float2 fa = make_float2(g4 * co, -g4 * so);
    const float2 fb = cmul(fa, fc);
    const float2 da = cmul(make_float2(4.0f * fmaf(omL, co, so), -4.0f * omL * so), fc);
    const float2 db = cadd(cmul(da, fc), cmul(fa, make_float2(fc.y, -fc.x)));
    // links 12, 23, 31, 21, 32, 13: arm, spacecraft, sign of k.r
    const int arm[6] = {0, 1, 2, 0, 1, 2};
    const int scq[6] = {0, 1, 2, 1, 2, 0};
    const float sg[6] = {1.f, 1.f, 1.f, -1.f, -1.f, -1.f};
    float pp[3], cc[3];
    float2 A[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        pp[a] = fmaf(rv[a], rv[a], -ru[a] * ru[a]);
        cc[a] = 2.0f * ru[a] * rv[a];
        A[a] = make_float2(fmaf(pp[a], B.DPf.x, cc[a] * B.DCf.x), fmaf(pp[a], B.DPf.y, cc[a] * B.DCf.y));
    }
    float2 gE[6], G[6];
    float dl[6], hh[6];
#pragma unroll
    for (int q = 0; q < 6; q++) {
        const int s = scq[q], a = arm[q];
        hh[q] = 0.5f * fmaf(sg[q], kd[a], 1.0f);
        const float av = fo[s] * hh[q];
        float S, C, dS;
        sinc_cos_d_f(av, S, C, dS);
        const float t = 0.25f * S;
        gE[q] = cmul(make_float2(t * C, -t * av * S), Es[s]);
        G[q] = cmul(gE[q], A[a]);
        dl[q] = dS / S;
    }
    // X, Y, Z of six link values with the factors (f1, f2), then A and E
    auto combine = [&](const float2 (&L)[6], float2 f1, float2 f2, float2 &oA, float2 &oE) {
        const float2 X = cadd(cmul(f1, csub(L[3], L[2])), cmul(f2, csub(L[0], L[5])));
        const float2 Y = cadd(cmul(f1, csub(L[4], L[0])), cmul(f2, csub(L[1], L[3])));
        const float2 Z = cadd(cmul(f1, csub(L[5], L[1])), cmul(f2, csub(L[2], L[4])));
        oA = make_float2((Z.x - X.x) * is2, (Z.y - X.y) * is2);
        oE = make_float2((X.x - 2.f * Y.x + Z.x) * is6, (X.y - 2.f * Y.y + Z.y) * is6);
    };
    {
        float2 L[6];
#pragma unroll
        for (int q = 0; q < 6; q++) L[q] = make_float2(gE[q].x * pp[arm[q]], gE[q].y * pp[arm[q]]);
        combine(L, fa, fb, outA[0], outE[0]);
#pragma unroll
        for (int q = 0; q < 6; q++) L[q] = make_float2(gE[q].x * cc[arm[q]], gE[q].y * cc[arm[q]]);
        combine(L, fa, fb, outA[1], outE[1]);
    }
    // d omL / d(f0 T, fdot T^2, fddot T^3) multiplies the (da, db) combination of G
    float2 wA, wE;
    combine(G, da, db, wA, wE);
    const float tau_m = tf * iT;
    const float dom[3] = {ifs * iT, ifs * iT * tau_m, 0.5f * ifs * iT * tau_m * tau_m};
    // frequency tangents: d fonfs_s = {1, tau, tau^2/2} ifs / T, d phase_s = -{2 pi tau, pi tau^2, pi/3 tau^3}
#pragma unroll
    for (int m = 0; m < 3; m++) {
        float2 L[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
            const int s = scq[q];
            const float x = tau[s];
            const float dfo = m == 0 ? ifs * iT : m == 1 ? ifs * iT * x : 0.5f * ifs * iT * x * x;
            const float dph = m == 0 ? -TWO_PI_F * x : m == 1 ? -PI_F * x * x : -(PI_F / 3.0f) * x * x * x;
            const float dav = hh[q] * dfo;
            L[q] = cmul(G[q], make_float2(dl[q] * dav, -(dav + dph)));
        }
        float2 oA, oE;
        combine(L, fa, fb, oA, oE);
        outA[2 + m] = make_float2(fmaf(dom[m], wA.x, oA.x), fmaf(dom[m], wA.y, oA.y));
        outE[2 + m] = make_float2(fmaf(dom[m], wE.x, oE.x), fmaf(dom[m], wE.y, oE.y));
    }
    // sky angles: d/dlam (du = -ct v, dv = ct u - st k, dk = st v),
    //             d/dbeta (du = -k, dv = 0, dk = u);
    // per spacecraft d kP moves phase_s by 2 pi f d kP and fonfs_s by
    // -(fdot + fddot xi)/fstar d kP
#pragma unroll
    for (int m = 0; m < 2; m++) {
        float2 L[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
            const int s = scq[q], a = arm[q];
            const float dkP = m == 0 ? dkPl[s] : dkPb[s];
            const float dfo = fmaf(Gx.gf1, xs[s], Gx.gf0) * dkP;
            const float dph = TWO_PI_F * fo[s] * fstarf * dkP;
            const float dkd = m == 0 ? Gx.st * rv[a] : ru[a];
            const float dav = fmaf(hh[q], dfo, 0.5f * sg[q] * fo[s] * dkd);
            float dpp, dcc;
            if (m == 0) {
                const float dru = -Gx.ct * rv[a], drv = fmaf(Gx.ct, ru[a], -Gx.st * kd[a]);
                dpp = 2.0f * fmaf(rv[a], drv, -ru[a] * dru);
                dcc = 2.0f * fmaf(dru, rv[a], ru[a] * drv);
            } else {
                dpp = 2.0f * ru[a] * kd[a];
                dcc = -2.0f * kd[a] * rv[a];
            }
            const float2 dA = make_float2(fmaf(dpp, B.DPf.x, dcc * B.DCf.x), fmaf(dpp, B.DPf.y, dcc * B.DCf.y));
            L[q] = cadd(cmul(G[q], make_float2(dl[q] * dav, -(dav + dph))), cmul(gE[q], dA));
        }
        combine(L, fa, fb, outA[5 + m], outE[5 + m]);
    }
}

struct FisherParams {
    KParams K;
    double *fisher;                // (num_bin, 9, 9) FP64, row-major per binary
};

__global__ void __launch_bounds__(kBlock, 2) fisher_kernel(const FisherParams FP)
{
    using V = float2;
    const KParams &K = FP.K;
    extern __shared__ __align__(16) unsigned char smem[];
    Bin *bins = reinterpret_cast<Bin *>(smem);
    GradExtra *gxs = reinterpret_cast<GradExtra *>(smem + sizeof(Bin) * K.maxP);
    double *red = reinterpret_cast<double *>(smem + (sizeof(Bin) + sizeof(GradExtra)) * K.maxP);
    V *buf = reinterpret_cast<V *>(smem + (sizeof(Bin) + sizeof(GradExtra)) * K.maxP +
                                   sizeof(double) * kFisherAcc * 2 * kMaxPack);
    __shared__ int s_tile;

    const gbx_wave_args &a = K.a;
    const int tid = threadIdx.x;
    const int ntiles = a.tiles ? a.ntiles : (a.num_bin + K.P - 1) / K.P;
    const float ifs = (float)(1.0 / K.fstar);
    const float fstarf = (float)K.fstar;
    const float Loc = (float)(1.0 / (kTwoPi * K.fstar));
    const float iT = (float)(1.0 / a.T);
    const Bin *wsb = static_cast<const Bin *>(a.workspace);
    const GradExtra *wsg = reinterpret_cast<const GradExtra *>(wsb + a.num_bin);
    constexpr int R2 = 2 * kFisherRows;
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
        const int maxcnt = tile_pack(a.tile, lg, 1);
        if (tab == nullptr || cnt < 1 || cnt > maxcnt || first < 0 || first + cnt > a.num_bin ||
            (cnt << lg) > K.maxS) {
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
        for (int m = tid; m < S; m += kBlock) {
            const int p = m >> lg, n = m & (N - 1);
            float2 oA[kFisherRows], oE[kFisherRows];
            slow_tangent_mixed(bins[p], gxs[p], n, N, stepd, Loc, tab, ifs, fstarf, iT, oA, oE);
            const int sn = swz(n, lg);
#pragma unroll
            for (int r = 0; r < kFisherRows; r++) {
                buf[(size_t)(p * R2 + 2 * r) * N + sn] = oA[r];
                buf[(size_t)(p * R2 + 2 * r + 1) * N + sn] = oE[r];
            }
        }
        __syncthreads();
        fft_dif<float>(buf, R2 * cnt, lg);

        const int Tpb = kBlock / maxcnt;
        const int width = Tpb < 32 ? Tpb : 32;
        const int p = tid / Tpb;
        const int i0 = tid - p * Tpb;
        float acc[kFisherAcc];
#pragma unroll
        for (int k = 0; k < kFisherAcc; k++) acc[k] = 0.0f;
        if (p < cnt && bins[p].valid) {
            const Bin &B = bins[p];
            const GradExtra &Gx = gxs[p];
            const float2 DP = B.DPf, DC = B.DCf;
            const float2 dPi = make_float2((float)Gx.dDPi.x, (float)Gx.dDPi.y);
            const float2 dCi = make_float2((float)Gx.dDCi.x, (float)Gx.dDCi.y);
            const float2 dPp = make_float2((float)Gx.dDPp.x, (float)Gx.dDPp.y);
            const float2 dCp = make_float2((float)Gx.dDCp.x, (float)Gx.dDCp.y);
            // d ln scale / d (f0 T)
            const float2 lsf = make_float2((float)(Gx.dlnsc_f0.x / a.T), (float)(Gx.dlnsc_f0.y / a.T));
            bool out = false;
            for (int i = i0; i < N; i += Tpb) {
                const int j = B.start + i;
                if (j < 0 || j >= K.L) {
                    out = true;
                    continue;
                }
                const int sp = swz(bitrev((i + (N >> 1)) & (N - 1), lg), lg);
                const size_t jn = (size_t)B.ni * K.L + j;
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    const double Sc = __ldg((c == 0 ? K.A_psd : K.E_psd) + jn);
                    const float w = __frcp_rn(d2f_scaled(Sc, B.eS));
                    float2 row[kFisherRows];
#pragma unroll
                    for (int r = 0; r < kFisherRows; r++) row[r] = buf[(size_t)(p * R2 + 2 * r + c) * N + sp];
                    const float2 yh = cadd(cmul(DP, row[0]), cmul(DC, row[1]));
                    // amp, f0, fdot, fddot, phi0, iota, psi, lam, beta
                    float2 D[kFisherPar];
                    D[0] = yh;
                    D[1] = cadd(row[2], cmul(lsf, yh));
                    D[2] = row[3];
                    D[3] = row[4];
                    D[4] = make_float2(-yh.y, yh.x);
                    D[5] = cadd(cmul(dPi, row[0]), cmul(dCi, row[1]));
                    D[6] = cadd(cmul(dPp, row[0]), cmul(dCp, row[1]));
                    D[7] = row[5];
                    D[8] = row[6];
                    int k = 0;
#pragma unroll
                    for (int u = 0; u < kFisherPar; u++) {
                        const float2 wu = make_float2(w * D[u].x, w * D[u].y);
#pragma unroll
                        for (int v = u; v < kFisherPar; v++, k++)
                            acc[k] = fmaf(wu.x, D[v].x, fmaf(wu.y, D[v].y, acc[k]));
                    }
                }
            }
            if (out) flag(a.status, GBX_FLAG_WINDOW);
        }
        // float-pair trees within groups, then per binary over its groups
        float2 *red2 = reinterpret_cast<float2 *>(red);
        double *tsum = red + kFisherAcc * kMaxPack;
        {
            const bool leader = (tid & (width - 1)) == 0;
            const int g = tid / width;
#pragma unroll
            for (int k = 0; k < kFisherAcc; k++) {
                dfl x = {acc[k], 0.f};
                for (int o = width >> 1; o > 0; o >>= 1) {
                    dfl y = {__shfl_xor_sync(0xffffffffu, x.h, o), __shfl_xor_sync(0xffffffffu, x.l, o)};
                    x = df_add(x, y);
                }
                if (leader) red2[kFisherAcc * g + k] = make_float2(x.h, x.l);
            }
        }
        __syncthreads();
        {
            const int per = Tpb / width;
            for (int t = tid; t < cnt * kFisherAcc; t += kBlock) {
                const int q = t / kFisherAcc, k = t - q * kFisherAcc;
                dfl x = {0.f, 0.f};
                for (int g = q * per; g < (q + 1) * per; g++) {
                    const float2 y = red2[kFisherAcc * g + k];
                    x = df_add(x, dfl{y.x, y.y});
                }
                tsum[t] = (double)x.h + (double)x.l;
            }
        }
        __syncthreads();
        for (int t = tid; t < cnt * kFisherPar * kFisherPar; t += kBlock) {
            const int q = t / (kFisherPar * kFisherPar);
            const int ij = t - q * kFisherPar * kFisherPar;
            const int i = ij / kFisherPar, j = ij - i * kFisherPar;
            const Bin &B = bins[q];
            if (B.b < 0) continue;
            const int u = min(i, j), v = max(i, j);
            // index of (u, v) in the packed upper triangle
            const int k = u * kFisherPar - u * (u - 1) / 2 + (v - u);
            // d/d amp = (1/amp) d/d ln amp; d/d f0 = T d/d(f0 T), fdot T^2, fddot T^3
            auto unit = [&](int r) {
                const double T = a.T;
                return r == 0 ? 1.0 / a.params[B.b] : r == 1 ? T : r == 2 ? T * T
                     : r == 3 ? T * T * T : 1.0;
            };
            const double s4 = 4.0 * K.df * exp2_int(B.eS) * (B.scale.x * B.scale.x + B.scale.y * B.scale.y);
            const double f = s4 * unit(u) * unit(v) * tsum[q * kFisherAcc + k];
            FP.fisher[(size_t)B.b * kFisherPar * kFisherPar + ij] = B.valid ? f : 0.0;
        }
        __syncthreads();
    }
}
