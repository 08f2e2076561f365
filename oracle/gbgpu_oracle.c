/*
 * CPU oracle for the GBGPU native kernels -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the two native loops of the reference:
 *   get_ll      gbgpu/cutils/gbgpu_utils.cu:124-185
 *   fill_global gbgpu/cutils/gbgpu_utils.cu:54-101
 * Complex numbers are interleaved double[2] (the layout of the reference's
 * gcmplx::complex<double>, gbgpu/cutils/global.h:66).  The arithmetic follows
 * the reference's operation order exactly (complex product a*c - b*d,
 * a*d + b*c; division of each component by the PSD; sequential sum over
 * i = 0..M-1, channel A before E; final scaling by (4 df)), and the library
 * is built with -ffp-contract=off so that no FMA contraction changes the
 * rounding.  Only tests and the CPU baseline of the benchmark load this file.
 *
 * The parallel variants split the binary loop over OpenMP threads; every
 * binary is still summed by one thread in the reference order, so their
 * results are bit-identical to the serial ones.
 */
#include <stddef.h>

static void ll_one(double *d_h, double *h_h, const double *A_t, const double *E_t,
                   const double *A_d, const double *E_d, const double *A_p,
                   const double *E_p, double df, const int *start_ind, int M,
                   int num_bin, const int *data_index, const int *noise_index,
                   int data_length, int b)
{
    const int start = start_ind[b];
    const long doff = (long)data_index[b] * data_length;
    const long noff = (long)noise_index[b] * data_length;
    double dh_re = 0.0, dh_im = 0.0, hh_re = 0.0, hh_im = 0.0;
    for (int i = 0; i < M; i++) {
        const long j = (long)start + i;
        const double SA = A_p[noff + j];
        const double SE = E_p[noff + j];
        const double hAr = A_t[2 * ((long)i * num_bin + b)];
        const double hAi = A_t[2 * ((long)i * num_bin + b) + 1];
        const double hEr = E_t[2 * ((long)i * num_bin + b)];
        const double hEi = E_t[2 * ((long)i * num_bin + b) + 1];
        const double dAr = A_d[2 * (doff + j)];
        const double dAi = -A_d[2 * (doff + j) + 1];   /* conj(d_A) */
        const double dEr = E_d[2 * (doff + j)];
        const double dEi = -E_d[2 * (doff + j) + 1];   /* conj(d_E) */
        double x, y;
        /* <d|h> */
        x = dAr * hAr - dAi * hAi; y = dAr * hAi + dAi * hAr;
        dh_re += x / SA; dh_im += y / SA;
        x = dEr * hEr - dEi * hEi; y = dEr * hEi + dEi * hEr;
        dh_re += x / SE; dh_im += y / SE;
        /* <h|h> */
        x = hAr * hAr - (-hAi) * hAi; y = hAr * hAi + (-hAi) * hAr;
        hh_re += x / SA; hh_im += y / SA;
        x = hEr * hEr - (-hEi) * hEi; y = hEr * hEi + (-hEi) * hEr;
        hh_re += x / SE; hh_im += y / SE;
    }
    const double s = 4. * df;
    d_h[2 * b] = s * dh_re; d_h[2 * b + 1] = s * dh_im;
    h_h[2 * b] = s * hh_re; h_h[2 * b + 1] = s * hh_im;
}

void oracle_get_ll(double *d_h, double *h_h, const double *A_t, const double *E_t,
                   const double *A_d, const double *E_d, const double *A_p,
                   const double *E_p, double df, const int *start_ind, int M,
                   int num_bin, const int *data_index, const int *noise_index,
                   int data_length)
{
    for (int b = 0; b < num_bin; b++)
        ll_one(d_h, h_h, A_t, E_t, A_d, E_d, A_p, E_p, df, start_ind, M, num_bin,
               data_index, noise_index, data_length, b);
}

void oracle_get_ll_par(double *d_h, double *h_h, const double *A_t, const double *E_t,
                       const double *A_d, const double *E_d, const double *A_p,
                       const double *E_p, double df, const int *start_ind, int M,
                       int num_bin, const int *data_index, const int *noise_index,
                       int data_length)
{
#pragma omp parallel for schedule(static)
    for (int b = 0; b < num_bin; b++)
        ll_one(d_h, h_h, A_t, E_t, A_d, E_d, A_p, E_p, df, start_ind, M, num_bin,
               data_index, noise_index, data_length, b);
}

void oracle_fill_global(double *A_g, double *E_g, const double *A_t, const double *E_t,
                        const int *start_ind, int M, int num_bin,
                        const int *group_index, int data_length)
{
    for (int b = 0; b < num_bin; b++) {
        const int start = start_ind[b];
        const long goff = (long)group_index[b] * data_length;
        for (int i = 0; i < M; i++) {
            const long j = (long)start + i;
            if (j >= data_length || j < 0)
                continue;
            const long t = 2 * ((long)i * num_bin + b);
            A_g[2 * (goff + j)] += A_t[t];
            A_g[2 * (goff + j) + 1] += A_t[t + 1];
            E_g[2 * (goff + j)] += E_t[t];
            E_g[2 * (goff + j) + 1] += E_t[t + 1];
        }
    }
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
