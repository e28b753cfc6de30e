// numerics.cpp -- small host-side numerics: tridiagonal eigensolver, continued fraction,
// reference start vector, CUDA error mapping.
#include <cmath>
#include <limits>
#include <random>

#include "esc_internal.h"

namespace esc {

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Implicit QL iteration with Wilkinson-type shifts on a real symmetric tridiagonal matrix
// (Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11, 293 (1968)).  Replaces LAPACK zheev
// on the Hermitian tridiagonal of DynLanczosSolver::TriDiag (src/DynLanczosSolver.h:371-414):
// the Lanczos alpha are real up to rounding (zheev ignores the imaginary part of the diagonal)
// and the beta are real, so the real symmetric problem is the same problem.
bool tridiag_eig(int n, std::vector<double>& d, std::vector<double> e, std::vector<double>* z) {
    if (n <= 0) return true;
    e.resize(n);
    e[n - 1] = 0.0;
    if (z) {
        z->assign((size_t)n * n, 0.0);
        for (int i = 0; i < n; i++) (*z)[(size_t)i * n + i] = 1.0;
    }
    const double eps = std::numeric_limits<double>::epsilon();
    for (int l = 0; l < n; l++) {
        for (int sweep = 0;; sweep++) {
            int m = l;
            while (m < n - 1 && std::fabs(e[m]) > eps * (std::fabs(d[m]) + std::fabs(d[m + 1]))) m++;
            if (m == l) break;
            if (sweep >= 80) return false;
            // shift from the leading 2x2 block
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
            double s = 1.0, c = 1.0, p = 0.0;
            bool underflow = false;
            for (int i = m - 1; i >= l; i--) {
                const double f = s * e[i], b = c * e[i];
                r = std::hypot(f, g);
                e[i + 1] = r;
                if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; underflow = true; break; }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
                if (z) {
                    double* zi = z->data() + (size_t)i * n;
                    double* zj = zi + n;
                    for (int k = 0; k < n; k++) {
                        const double t = zj[k];
                        zj[k] = s * zi[k] + c * t;
                        zi[k] = c * zi[k] - s * t;
                    }
                }
            }
            if (underflow) continue;
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    // ascending order, eigenvectors follow (insertion sort: n <= a few thousand)
    for (int i = 1; i < n; i++) {
        int j = i;
        while (j > 0 && d[j - 1] > d[j]) {
            std::swap(d[j - 1], d[j]);
            if (z) {
                double* a = z->data() + (size_t)(j - 1) * n;
                double* b = a + n;
                for (int k = 0; k < n; k++) std::swap(a[k], b[k]);
            }
            j--;
        }
    }
    return true;
}

cplx cf_eval(const double* a, const double* b, int n, cplx z) {
    if (n <= 0) return cplx(0.0, 0.0);
    cplx t(0.0, 0.0);
    for (int k = n - 1; k >= 1; k--) t = (b[k] * b[k]) / (z - a[k] - t);
    return (b[0] * b[0]) / (z - a[0] - t);
}

// src/DynLanczosSolver.h:465-474 with the generator of src/ParametersEngine.h:19,62-64,152-154.
// uniform_real_distribution<double>(0,1) on a 64-bit engine draws once: double(x - min) / 2^64.
void ref_uniform_start(int seed, int64_t D, cplx* out) {
    std::mt19937_64 g((unsigned long long)seed);
    auto u = [&]() {
        double r = double(g() - std::mt19937_64::min()) / 18446744073709551616.0;
        return r < 1.0 ? r : std::nextafter(1.0, 0.0);
    };
    for (int64_t i = 0; i < D; i++) {
        const double re = -1.0 + u() * 2.0;
        const double im = -1.0 + u() * 2.0;
        out[i] = cplx(re, im);
    }
}

}  // namespace esc
