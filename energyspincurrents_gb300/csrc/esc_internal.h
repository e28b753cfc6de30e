// esc_internal.h -- shared declarations of the GB300 Lanczos ED library (host C++ + CUDA).
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/esc.h"

namespace esc {

constexpr int MAX_SITES = 40;     // 2^40 complex64 = 8.8 TB: far beyond one GPU, so never binding
constexpr int MAX_BONDS = 96;     // honeycomb: 3N/2 = 48 at N = 32
constexpr int MAX_TERMS = 256;    // operator strings (spin-current total: 6N terms)
constexpr int MAX_COLS = 16;      // columns of one batched H.V launch

typedef std::complex<double> cplx;

// ---------------------------------------------------------------------------------------------
// Device-side model, passed by value as a __grid_constant__ kernel parameter (so that several
// handles with different models can coexist; no __constant__ globals).
//
// Off-diagonal bond term (i,j): out[k] += c(k) * in[k ^ mask], c = bits i,j equal ? ceq : cdiff.
//   Built from per-bond couplings (kx, ky, kz) as ceq = (kx - ky)/4, cdiff = (kx + ky)/4, which
//   reproduces the reference's S^x S^x (1/4) and S^y S^y (-1/4 equal, +1/4 differ) matrix
//   elements (src/Hamiltonian.h:113-158) and adds J S.S where enabled.
// Diagonal bond term: dz * (equal ? +1/4 : -1/4) (src/Hamiltonian.h:344-360).
// Field: out[k] += (Bx/2 + i By/2 * (bit_s(k) ? +1 : -1)) in[k ^ 2^s]  (:167-198)
//        diag   += Bz/2 * (N - 2 popcount(k))                         (:364-375)
// ---------------------------------------------------------------------------------------------
struct DevBond {
    unsigned long long mask;
    double ceq, cdiff;
};
struct DevDiagBond {
    unsigned long long mask;
    double dz;
};
struct DevModel {
    int N;
    int nb;          // off-diagonal bonds
    int nd;          // diagonal bonds
    int pad;
    double fx, fy, fz;   // Bx/2, By/2, Bz/2
    DevBond b[MAX_BONDS];
    DevDiagBond d[MAX_BONDS];
    // float copies for the complex64 path (GB300 runs FP64 and FP64<->FP32 conversions at a small
    // fraction of the FP32 rate, so the float kernels must not touch a double per term)
    float fxf, fyf, fzf, padf;
    float ceqf[MAX_BONDS], cdifff[MAX_BONDS];
    float dqf[MAX_BONDS];   // dz/4
    // device words of the slab-pair passes (hv_tiled.cu): [0] error flag, [SLAB_CNT0 ..] per-slab
    // counters; NULL: passes are never paired (a model that no handle owns)
    unsigned* slab_sync;
};
void fill_float_copies(DevModel& m);
// Per-column field (batched H.V with one field per column).
struct DevFields {
    double fx[MAX_COLS], fy[MAX_COLS], fz[MAX_COLS];
    float fxf[MAX_COLS], fyf[MAX_COLS], fzf[MAX_COLS];
};
// Columns of one tiled H.V launch sequence: column c reads in + c ld and writes out + c ld with the
// field f[c]; dotp (may be NULL) receives the alpha partials sum conj(in) out of every column from
// the last pass, (re, im) at dotp[(c * G + b) * 2] for b < G (G returned by the launcher).
struct DevCols {
    long long ld = 0;
    int ncols = 1;
    int col0 = 0;            // global index of column 0 in the layout of dotp (launches over a column range)
    DevFields f{};
    double* dotp = nullptr;
};
DevCols single_column(const DevModel& m);

// Operator = sum of terms; term t = coef * f_{n-1} ... f_0 (f_0 applied first), each factor a
// single-site S^x/S^y/S^z.  Gather form: out[k] += coef * phi_t(k0) * in[k0], k0 = k ^ flip.
struct DevOp {
    int nt;
    int pad;
    unsigned long long flip[MAX_TERMS];
    unsigned int fac[MAX_TERMS];   // bits 0-1 nf; factor f at bits 2+8f: 6 bits site, 2 bits op (1 x, 2 y, 3 z)
    double cre[MAX_TERMS], cim[MAX_TERMS];
    float cref[MAX_TERMS], cimf[MAX_TERMS];
};

// ---------------------------------------------------------------------------------------------
// Host-side model
// ---------------------------------------------------------------------------------------------
struct Bond {
    int i, j;
    char type;                // 'x' 'y' 'z' (honeycomb column) or 'c' (chain)
    double kx, ky, kz;        // coupling of S^aS^a on this bond (incl. J)
};

struct Lattice {
    int N = 0, ncol = 0;
    std::vector<int> neigh;   // N x 3, -1 = none
    std::vector<int> indx, indy;
};

struct Params;  // = esc_params

void build_lattice(const esc_params& p, Lattice& L);
void build_bonds(const esc_params& p, const Lattice& L, std::vector<Bond>& bonds);
DevModel make_dev_model(const esc_params& p, const Lattice& L, const std::vector<Bond>& bonds,
                        double Bx, double By, double Bz);

// ---------------------------------------------------------------------------------------------
// Tiled H.v (hv_tiled.cu, planner.cpp)
// ---------------------------------------------------------------------------------------------
struct Plan {
    int N = 0, T = 0, c = 0;
    std::vector<int> perm;                 // site -> bit position of the internal basis index
    std::vector<std::vector<int>> tiles;   // per pass: sorted tile bit positions (include [0,c))
};
Plan make_plan(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts);
// Same covering with no relabelling: the shared sites are 0..c-1 and tiles are sets of reference bits.
Plan make_plan_reference_order(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts);

constexpr int MAX_PTERMS = 96;
struct DevPass {
    int Tp, c, nrest, nbond, nfield, diag, accumulate, pad;
    unsigned long long tabLo[64], tabHi[64];   // run index -> global offset (low / high 6 bits)
    unsigned char rest[MAX_SITES];             // bit positions of the tile number, ascending
    unsigned int blm[MAX_PTERMS];              // bond masks in tile-local bits
    double ceq[MAX_PTERMS], cdiff[MAX_PTERMS];
    float ceqf[MAX_PTERMS], cdifff[MAX_PTERMS];   // the same in float for the complex64 path
    unsigned int flm[MAX_SITES];               // field-term masks in tile-local bits
    // fast kernel (512 threads, thread t owns tile states t + 512 j): parity of the bits of
    // (512 j) under each term mask, bit j
    unsigned int bjpar[MAX_PTERMS];
    unsigned int fjbit[MAX_SITES];
    // Register-grouped form (complex64 kernel): the terms ordered by their thread-bit mask
    // (tile-local bits below tb_bits).  A thread loads the partners of a group once -- its E
    // register states, with the group's thread bits flipped -- and applies every term of the group
    // from registers; the term's register-bit mask (local bits tb_bits..) selects the register.
    int ngroup, nterm;
    unsigned short glo[MAX_PTERMS + MAX_SITES];   // thread-bit mask of group g
    unsigned char gnt[MAX_PTERMS + MAX_SITES];    // terms in group g
    unsigned char gk[MAX_PTERMS + MAX_SITES];     // term code: bond = register mask (0..31); field = 33 + register bit, 32 = thread-bit field
    float ga[MAX_PTERMS + MAX_SITES], gb[MAX_PTERMS + MAX_SITES];   // bond: ceq, cdiff
    int jit;      // kernel specialised for this pass at run time (hv_jit.cu), -1: none
    int stages;   // complex64 pass: 2 or 3 tile buffers per CTA, 4 = 2 + staged epilogue loads
    int tb_bits;  // complex64 grouped pass: log2 of the threads per tile (9: 512, 8: 256, 7: 128)
    // Slab pair (complex64, one column): pair = 1 marks the first pass of a pair with the next pass
    // (both run in one launch, slab by slab); slab_bits = bits spanned by the two tiles together.
    int pair, slab_bits;
    int jit_pair;  // specialised pair kernel of this pass and the next (hv_jit.cu), -1: none
};
// Slab pairs: consecutive passes whose tiles together span at most SLAB_MAX_BITS bits can run as
// one launch over slabs of 2^slab_bits states (2^21 complex64 states = 16 MB: the slab's input,
// partial result and diagonal can stay in the L2 cache between the two passes).  From
// SLAB_MIN_SITES sites on the planner orders the passes in such pairs and the self-tuner times the
// paired launches against the single ones; ESC_SLAB_PAIRS=1 pairs at any size without tuning, =0
// never.
constexpr int SLAB_MIN_SITES = 27;
constexpr int SLAB_MAX_BITS = 21;
constexpr int SLAB_CNT0 = 32;   // first counter word of DevModel::slab_sync
// -1: no environment override, 0: pairs off, 1: pairs at every size
int slab_pairs_env();
// Slab-pair launches made by this process so far (a handle checks its error flag when it changed).
unsigned long long slab_pair_launches();
// Marks the slab pairs of a pass list (DevPass::pair, ::slab_bits): consecutive passes whose
// tiles span at most SLAB_MAX_BITS of the N bits together, greedily from the first pass.
void mark_pairs(std::vector<DevPass>& ps, int N);
// A pair kernel exists for passes a, b: the specialised one (a.jit_pair), or the ahead-of-time one
// (512 threads per tile in both, 4096- or 8192-state tiles).
inline bool pair_launchable(const DevPass& a, const DevPass& b) {
    return a.jit_pair >= 0 || (a.tb_bits == 9 && b.tb_bits == 9 && (a.Tp == 12 || a.Tp == 13));
}
// Words of DevModel::slab_sync for a basis of N sites.
inline size_t slab_sync_words(int N) { return (size_t)SLAB_CNT0 + (N > 12 ? (size_t)1 << (N - 12) : 1); }
// Orders the passes of a plan so that consecutive pairs span few bits (planner.cpp); applied
// from SLAB_MIN_SITES sites on, or at any size when ESC_SLAB_PAIRS is set.
void order_for_pairs(Plan& P);
// Builds one DevPass per plan pass from the relabelled model; throws if a term fits no tile.
// balance: term -> pass assignment (0 first eligible pass, 1 balanced, -1 from ESC_PASS_BALANCE);
// stages: tile buffers of the complex64 passes (0: from ESC_STAGES, default 2).
// tb_bits: threads per tile of the grouped complex64 pass, 2^tb_bits (7..9; 0: ESC_TB_BITS, else 9).
std::vector<DevPass> make_passes(const Plan& P, const DevModel& m, int balance = -1, int stages = 0, int tb_bits = 0);
}  // namespace esc
namespace escdev { struct PassTab; struct PairTab; }
namespace esc {
// Run-time specialisation of the complex64 passes (hv_jit.cu): compiles one kernel per eligible
// pass with its term groups written out, and one per slab pair of two such passes, for the
// current device, and sets DevPass::jit and ::jit_pair.  Returns false (passes unchanged) with a
// message if NVRTC or the module load fails.
bool jit_compile(std::vector<DevPass>& passes, std::string& err);
// The CUDA source jit_compile hands to NVRTC; which (optional) receives the pass index of each
// kernel esc_jit_pass<k>, pairs the first pass of each kernel esc_jit_pair<q>.
std::string jit_source(const std::vector<DevPass>& passes, std::vector<int>* which, std::vector<int>* pairs = nullptr);
// Launches the specialised kernel of pass p; returns its grid size.
int jit_launch(const DevPass& p, const escdev::PassTab& pt, const void* diag, const void* in, void* out, int64_t D,
               int sms, cudaStream_t s, const int* active);
escdev::PassTab make_pass_tab(const DevPass& p, const DevModel& m, const DevCols* cols = nullptr, double* dotp = nullptr);
// Slab-pair table of passes a and b (a.pair set) over N sites; sync = DevModel::slab_sync.
escdev::PairTab make_pair_tab(const DevPass& a, const DevPass& b, int N, unsigned* sync);
// Launches the specialised pair kernel of a (a.jit_pair) cooperatively; returns its grid.
int jit_pair_launch(const DevPass& a, const escdev::PassTab& pa, const escdev::PassTab& pb, const escdev::PairTab& st,
                    const void* diag, const void* in, void* out, int64_t D, int sms, cudaStream_t s, const int* active);
// Default tile buffers per CTA of the complex64 passes (2; ESC_STAGES=3 for three).
int pass_stages();
// diag: precomputed diagonal of the bond terms (no field), R per state (launch_diag); may be NULL,
// then the diagonal is computed in the kernel.
// active (optional, device int): the launches do nothing when *active == 0 (batched recurrences).
template <typename R> void launch_hv_tiled(const DevModel& m, const std::vector<DevPass>& passes, const void* in,
                                           void* out, int64_t D, const void* diag, cudaStream_t s,
                                           const int* active = nullptr);
// Multi-column form: all active columns (device flags active[c], may be NULL) in one launch per
// pass; returns the number G of alpha partials per column written to cols.dotp (0 without dotp).
template <typename R> int launch_hv_cols(const DevModel& m, const DevCols& cols, const std::vector<DevPass>& passes,
                                         const void* in, void* out, int64_t D, const void* diag, cudaStream_t s,
                                         const int* active);
template <typename R> void launch_diag(const DevModel& m, void* diag, int64_t D, cudaStream_t s);
// host_sum = <v|H|v> (re, im) computed in FP64 pass by pass; S = storage precision of v.
template <typename S> void launch_energy(const DevModel& m, const std::vector<DevPass>& passes, const void* in,
                                         int64_t D, double* partials, int max_blocks, std::vector<double>& host_sum,
                                         cudaStream_t s);
// y += z[idx] * x  (real coefficient read from device memory)
template <typename R> void launch_axpy_dev(const void* x, void* y, const double* d_coef, int64_t n, cudaStream_t s);
// Basis permutation: out[j] = in[src(j)], src assembled bitwise from five 8-bit tables.
struct DevPerm {
    unsigned long long tab[5][256];
    int N;
    signed char sb[MAX_SITES];   // src bit of each dst bit
};
DevPerm make_perm_table(const std::vector<int>& bit_of_src_bit);   // tab maps dst index bits -> src index
template <typename R> void launch_permute(const DevPerm& p, const void* in, void* out, int64_t D, cudaStream_t s);

struct OpTerm {
    cplx coef;
    int nf;
    int site[3];
    char op[3];   // 'x' 'y' 'z'
};
// Throws std::invalid_argument for unknown operators / missing neighbours.
std::vector<OpTerm> operator_terms(int op, int site, const esc_params& p, const Lattice& L);
// perm (optional): site -> internal bit position
DevOp make_dev_op(const std::vector<OpTerm>& terms, const std::vector<int>* perm = nullptr);

// ---------------------------------------------------------------------------------------------
// Kernel launchers (kernels.cu).  R = double (complex128 vectors) or float (complex64 vectors).
// Reductions always accumulate in double and are deterministic: fixed grids, fixed trees.
// ---------------------------------------------------------------------------------------------
int red_blocks(int64_t n);
constexpr int RED_MAX_BLOCKS = 1216;   // 8 x 152 SMs

template <typename R> void launch_apply(const DevOp& op, const void* in, void* out, int64_t D, cudaStream_t s);

// dst (double2) = sum conj(a) b
template <typename R> void launch_dot(const void* a, const void* b, int64_t n, double* partials, double* dst,
                                      cudaStream_t s);
// dst (double) = |a|^2
template <typename R> void launch_nrm2(const void* a, int64_t n, double* partials, double* dst, cudaStream_t s);
// w = w - alpha*v - beta*u (alpha: double2 at d_alpha, beta = sqrt(*d_beta2), u may be NULL);
// then dst = |w|^2
template <typename R> void launch_lanczos_update(void* w, const void* v, const void* u, const double* d_alpha,
                                                 const double* d_beta2, int64_t n, double* partials, double* dst,
                                                 cudaStream_t s);
// out = in / sqrt(*d_nrm2)  (out may equal in)
template <typename R> void launch_scale_rsqrt(const void* in, void* out, const double* d_nrm2, int64_t n,
                                              cudaStream_t s);
// out = a*x + b*y  (complex scalars on host)
template <typename R> void launch_axpby(const void* x, const void* y, void* out, cplx a, cplx b, int64_t n,
                                        cudaStream_t s);
// r[j] = sum_k conj(L_j[k]) w[k], j < m; L_j at L + j*ld (elements).  r: m double2.
template <typename R> void launch_gemv_h(const void* L, int64_t ld, int m, const void* w, int64_t n,
                                         double* partials, int64_t partials_cap, double* r, cudaStream_t s);
// w[k] -= sum_j L_j[k] r[j]   (r: m double2 on device)
template <typename R> void launch_gemv_sub(const void* L, int64_t ld, int m, const double* r, void* w, int64_t n,
                                           cudaStream_t s);
// out[k] = sum_j L_j[k] z[j]  (z: m doubles on device, real)
template <typename R> void launch_lincomb(const void* L, int64_t ld, int m, const double* z, void* out, int64_t n,
                                          cudaStream_t s);
void launch_convert_c128_to_c64(const void* in, void* out, int64_t n, cudaStream_t s);
// unit vectors e_{j0} .. e_{j0+ncols-1} as ncols columns of D states (stride D)
template <typename R> void launch_unit_columns(void* out, int64_t D, int64_t j0, int ncols, cudaStream_t s);
void launch_convert_c64_to_c128(const void* in, void* out, int64_t n, cudaStream_t s);
template <typename R> void launch_start_normal(uint64_t seed, void* out, int64_t n, cudaStream_t s);

// Batched continued-fraction Lanczos (batched.cu).  Caller fills the pointers (device memory) and
// the per-column H.v callback; run() executes kmax iterations (CUDA graph if use_graph).
template <typename R>
struct CFBatch {
    int ncols = 0, kmax = 0;
    int64_t D = 0;
    double tol = 1e-10;
    bool use_graph = true;
    void* bufs = nullptr;        // 3 sets of ncols vectors; set 1 holds the start vectors on entry
    double* d_part = nullptr;    // ncols * 304 * 2 doubles
    double* d_alpha = nullptr;   // ncols * kmax * 2
    double* d_b2 = nullptr;      // ncols * (kmax + 1); [c][0] = |phi_c|^2
    int* d_active = nullptr;     // ncols
    int* d_it = nullptr;         // 1
    int* d_steps = nullptr;      // ncols (per-column step limit <= kmax)
    // start_it > 0 continues a recurrence at iteration start_it: prev = set start_it % 3, cur =
    // set (start_it + 1) % 3, alpha / b2 filled below start_it, active flags set by the caller
    int start_it = 0;
    // w = H cur for every active column; writes the alpha partials sum conj(cur) w of column c at
    // part[(c * G + b) * 2] and returns G (launch_hv_cols)
    std::function<int(const void* cur, void* w, const int* active, double* part, cudaStream_t)> hv_all;
    // optional, run (and captured) after the update of every iteration: w holds u_{it+1} of every
    // column, the iteration counter is at d_it
    std::function<void(const void* w, cudaStream_t)> after_update;
    void run(cudaStream_t s);
};
constexpr int CFB_GRID = 1216;   // blocks per column of the batched CF kernels (8 x 152 SMs)
// One-column helpers for the ground-state Lanczos on the CFBatch recurrence (device iteration
// counter d_it, column flag d_active[0]): L[it+1] = w, and gs += zc[it+1] w.
template <typename R> void launch_store_iter(const void* w, void* L, int64_t D, const int* d_it, const int* d_active,
                                             cudaStream_t s);
template <typename R> void launch_accum_iter(const void* w, void* gs, int64_t D, const int* d_it, const double* zc,
                                             const int* d_active, cudaStream_t s);

// ---------------------------------------------------------------------------------------------
// Host numerics
// ---------------------------------------------------------------------------------------------
// Symmetric tridiagonal eigenproblem (implicit QL); d: diagonal, e: off-diagonal (e[i] couples
// i,i+1).  Eigenvalues ascending in d; z (optional) n x n column-major.  Returns false on failure.
bool tridiag_eig(int n, std::vector<double>& d, std::vector<double> e, std::vector<double>* z);

// Continued fraction b0^2/(z - a0 - b1^2/(z - a1 - ...)).
cplx cf_eval(const double* a, const double* b, int n, cplx z);

// Reference start vector: mt19937_64(seed), generate_canonical<double,53> draws, re then im.
void ref_uniform_start(int seed, int64_t D, cplx* out);

// Sets the message that esc_last_error(NULL) returns on this thread.
void set_last_error(const std::string& msg);

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
void check_cuda(cudaError_t e, const char* what);
#define ESC_CUDA(x) ::esc::check_cuda((x), #x)

}  // namespace esc
