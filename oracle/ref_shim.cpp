// ref_shim.cpp -- C entry points over the reference's own C++ core, for
// validating the oracle restatement.  TEST INFRASTRUCTURE ONLY.
//
// The reference header software/core/libuap.hpp is NOT copied here: the
// recipe in oracle/Makefile compiles this file with -I pointing at the
// reference checkout, and the resulting library lands in oracle/_ref/
// (git-ignored).  The wrapped calls are uap::forward_fmc (libuap.hpp:109) and
// uap::misfit_and_gradient (libuap.hpp:169), exactly as the reference's
// pybind11 module software/python/_uap.cpp:25-55 calls them.
#include "libuap.hpp"

extern "C" {

int usct_ref_forward_fmc(const double* m, const int* dims, int ndim, double h, double dt, int nt,
                         const int* tx_lin, int n_tx, const int* rec_lin, int n_rec,
                         const double* wavelet, double* data) {
    uap::forward_fmc(m, dims, ndim, h, dt, nt, tx_lin, n_tx, rec_lin, n_rec, wavelet, data);
    return 0;
}

double usct_ref_misfit_and_gradient(const double* m, const int* dims, int ndim, double h, double dt,
                                    int nt, const int* tx_lin, int n_tx, const int* rec_lin,
                                    int n_rec, const double* wavelet, const double* dobs,
                                    double* grad, int misfit_type) {
    return uap::misfit_and_gradient(m, dims, ndim, h, dt, nt, tx_lin, n_tx, rec_lin, n_rec,
                                    wavelet, dobs, grad, misfit_type);
}

}  // extern "C"
