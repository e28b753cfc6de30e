// Test-only bridge from the LAPACK names the reference declares (src/DynLanczosSolver.h:17-21,
// src/Exactdiag.h:14-15, src/Observables.h:14) to the LP64 OpenBLAS that ships inside scipy's
// wheel (symbols scipy_zheev_ / scipy_dstev_).  Hidden Fortran string lengths are passed as 1.
#include <complex>
#include <cstddef>
extern "C" {
void scipy_zheev_(char*, char*, int*, std::complex<double>*, int*, double*, std::complex<double>*, int*, double*, int*, size_t, size_t);
void scipy_dstev_(char*, int*, double*, double*, double*, int*, double*, int*, size_t);
void zheev_(char* jobz, char* uplo, int* n, std::complex<double>* a, int* lda, double* w,
            std::complex<double>* work, int* lwork, double* rwork, int* info) {
    scipy_zheev_(jobz, uplo, n, a, lda, w, work, lwork, rwork, info, 1, 1);
}
void dstev_(char* jobz, int* n, double* d, double* e, double* z, int* ldz, double* work, int* info) {
    scipy_dstev_(jobz, n, d, e, z, ldz, work, info, 1);
}
}
