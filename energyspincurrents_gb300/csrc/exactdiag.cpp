// exactdiag.cpp -- Solver=ED: dense exact diagonalisation of small clusters on the device.
//
// Replaces ExactDiag + DynLanczosSolver::fillFromED (src/Exactdiag.h:36-81, src/DynLanczosSolver.h:
// 269-283; chosen in main.cpp:79-83).  The reference assembles the dense matrix from its COO lists
// (and leaves it uninitialised before adding them, src/Exactdiag.h:42) and calls LAPACK zheev; here
// the dense 2^N x 2^N complex128 matrix is built on the device, 16 columns at a time, as H applied
// to unit vectors by the tiled multi-column passes (so it is the same H as every other call), and
// diagonalised by cuSOLVER's Hermitian divide-and-conquer eigensolver.  cuSOLVER is loaded when ED
// is first asked for, so the library has no link-time dependency on it.  All 2^N eigenpairs then
// take the place of the Ritz pairs: Ritz-mode spectra sum over the exact spectrum, and the ground
// state is the lowest eigenvector.
#include <cusolverDn.h>
#include <dlfcn.h>

#include "abi_common.h"

namespace escabi {

namespace {

struct Solver {
    decltype(&::cusolverDnCreate) create = nullptr;
    decltype(&::cusolverDnDestroy) destroy = nullptr;
    decltype(&::cusolverDnSetStream) set_stream = nullptr;
    decltype(&::cusolverDnZheevd_bufferSize) buffer_size = nullptr;
    decltype(&::cusolverDnZheevd) zheevd = nullptr;
    bool ok = false;
};

const Solver& solver() {
    static Solver s = [] {
        Solver x;
        void* lib = nullptr;
        for (const char* name : {"libcusolver.so.12", "libcusolver.so.11", "libcusolver.so"})
            if ((lib = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
        if (!lib) return x;
        x.create = (decltype(x.create))dlsym(lib, "cusolverDnCreate");
        x.destroy = (decltype(x.destroy))dlsym(lib, "cusolverDnDestroy");
        x.set_stream = (decltype(x.set_stream))dlsym(lib, "cusolverDnSetStream");
        x.buffer_size = (decltype(x.buffer_size))dlsym(lib, "cusolverDnZheevd_bufferSize");
        x.zheevd = (decltype(x.zheevd))dlsym(lib, "cusolverDnZheevd");
        x.ok = x.create && x.destroy && x.set_stream && x.buffer_size && x.zheevd;
        return x;
    }();
    return s;
}

}  // namespace

constexpr int ED_MAX_SITES = 14;   // a 2^14 x 2^14 complex128 matrix is 4.3 GB

void exact_diag(esc_handle* h) {
    const int64_t D = h->D;
    if (h->N > ED_MAX_SITES)
        throw Fail(ESC_ERR_PARAM, "Solver=ED: at most " + std::to_string(ED_MAX_SITES) +
                                      " sites (the dense matrix has 4^N complex entries)");
    const Solver& S = solver();
    if (!S.ok) throw Fail(ESC_ERR_CUDA, "Solver=ED needs cuSOLVER (libcusolver.so) at run time");
    h->have_gs = h->have_basis = false;
    release_staging(h, 0);
    // dense H (column-major, internal basis order): column j = H e_j
    void* A = nullptr;
    void* E = nullptr;
    ESC_CUDA(cudaMalloc(&A, (size_t)D * D * 16));
    try {
        ESC_CUDA(cudaMalloc(&E, (size_t)esc::MAX_COLS * D * 16));
        esc::DevCols cols = esc::single_column(h->dm);
        cols.ld = D;
        for (int c = 1; c < esc::MAX_COLS; c++) {
            cols.f.fx[c] = cols.f.fx[0]; cols.f.fy[c] = cols.f.fy[0]; cols.f.fz[c] = cols.f.fz[0];
            cols.f.fxf[c] = cols.f.fxf[0]; cols.f.fyf[c] = cols.f.fyf[0]; cols.f.fzf[c] = cols.f.fzf[0];
        }
        const void* dg = diag_for(h, ESC_C128);
        for (int64_t j0 = 0; j0 < D; j0 += esc::MAX_COLS) {
            const int nc = (int)std::min<int64_t>(esc::MAX_COLS, D - j0);
            esc::launch_unit_columns<double>(E, D, j0, nc, h->stream);
            cols.ncols = nc;
            esc::launch_hv_cols<double>(h->dm, cols, h->passes, E, (char*)A + (size_t)j0 * D * 16, D, dg, h->stream,
                                        nullptr);
        }
        cudaFree(E);
        E = nullptr;
        // eigenpairs
        cusolverDnHandle_t sh = nullptr;
        if (S.create(&sh) != CUSOLVER_STATUS_SUCCESS) throw Fail(ESC_ERR_CUDA, "cusolverDnCreate failed");
        double* W = nullptr;
        void* work = nullptr;
        int* info = nullptr;
        auto cleanup = [&]() {
            if (W) cudaFree(W);
            if (work) cudaFree(work);
            if (info) cudaFree(info);
            S.destroy(sh);
        };
        try {
            S.set_stream(sh, h->stream);
            int lwork = 0;
            if (S.buffer_size(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)D, (cuDoubleComplex*)A, (int)D, nullptr,
                              &lwork) != CUSOLVER_STATUS_SUCCESS)
                throw Fail(ESC_ERR_CUDA, "cusolverDnZheevd_bufferSize failed");
            ESC_CUDA(cudaMalloc(&W, (size_t)D * sizeof(double)));
            ESC_CUDA(cudaMalloc(&work, (size_t)lwork * 16));
            ESC_CUDA(cudaMalloc(&info, sizeof(int)));
            if (S.zheevd(sh, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)D, (cuDoubleComplex*)A, (int)D, W,
                         (cuDoubleComplex*)work, lwork, info) != CUSOLVER_STATUS_SUCCESS)
                throw Fail(ESC_ERR_CUDA, "cusolverDnZheevd failed");
            int hinfo = 0;
            h->ritz.assign((size_t)D, 0.0);
            ESC_CUDA(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
            ESC_CUDA(cudaMemcpyAsync(h->ritz.data(), W, (size_t)D * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            sync(h);
            if (hinfo != 0)   // the reference's zheev failure (src/Exactdiag.h:104-107)
                throw Fail(ESC_ERR_NUMERIC, "diag: zheev: failed with info!=0 (info=" + std::to_string(hinfo) + ")");
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
    } catch (...) {
        if (E) cudaFree(E);
        cudaFree(A);
        throw;
    }
    // fillFromED: eigenvectors = the basis (column k = eigenvector k), eigenvalues = the Ritz values
    if (h->d_L) cudaFree(h->d_L);
    h->d_L = A;
    h->L_bytes = (size_t)D * D * 16;
    h->L_ld = D;
    h->nsteps = (int)D;
    h->exact = true;
    h->Z.clear();
    h->alpha.clear();
    h->beta.clear();
    ensure(h->d_gs, h->gs_bytes, (size_t)D * 16);
    ESC_CUDA(cudaMemcpyAsync(h->d_gs, A, (size_t)D * 16, cudaMemcpyDeviceToDevice, h->stream));   // Psi = Evec.col(0)
    h->basis_dt = ESC_C128;
    h->have_gs = h->have_basis = true;
    sync(h);
}

}  // namespace escabi

extern "C" esc_status esc_exact_diag(esc_handle* h, double* evals, void* gs_out, int flags) {
    using namespace escabi;
    if (!h) return finish(h, ESC_ERR_PARAM, "null argument");
    return guarded(h, [&]() {
        exact_diag(h);
        if (evals) std::copy(h->ritz.begin(), h->ritz.end(), evals);
        if (gs_out) {
            Staged g{nullptr, h->d_gs, h->D};
            unstage(h, g, gs_out, 1, h->D, ESC_C128, flags & ~ESC_ASYNC);
        }
    });
}
