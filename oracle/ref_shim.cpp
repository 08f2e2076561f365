// TEST INFRASTRUCTURE ONLY (oracle).  Gives C linkage to the reference's own
// get_ll_wrap / fill_global_wrap (gbgpu/cutils/gbgpu_utils.hh:6-13), which
// are compiled unmodified from gbgpu/cutils/gbgpu_utils.cu as C++ by
// oracle/Makefile.  cmplx is gcmplx::complex<double>, layout-compatible with
// interleaved double[2].
#include "gbgpu_utils.hh"

extern "C" void ref_get_ll(void *d_h, void *h_h, void *A_t, void *E_t,
                           void *A_d, void *E_d, void *A_p, void *E_p,
                           double df, void *start_ind, int M, int num_bin,
                           void *data_index, void *noise_index, int data_length)
{
    get_ll_wrap((cmplx *)d_h, (cmplx *)h_h, (cmplx *)A_t, (cmplx *)E_t,
                (cmplx *)A_d, (cmplx *)E_d, (double *)A_p, (double *)E_p, df,
                (int *)start_ind, M, num_bin, (int *)data_index,
                (int *)noise_index, data_length);
}

extern "C" void ref_fill_global(void *A_g, void *E_g, void *A_t, void *E_t,
                                void *start_ind, int M, int num_bin,
                                void *group_index, int data_length)
{
    fill_global_wrap((cmplx *)A_g, (cmplx *)E_g, (cmplx *)A_t, (cmplx *)E_t,
                     (int *)start_ind, M, num_bin, (int *)group_index,
                     data_length);
}
