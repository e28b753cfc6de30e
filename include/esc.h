/*
 * esc.h -- C ABI of the GB300 (sm_103a) Lanczos exact-diagonalisation library.
 *
 * Drop-in for the Lanczos path of fengshi96/EnergySpinCurrents ("LanczosCond"): the spin-1/2
 * Kitaev(-Heisenberg) honeycomb model (and the Heisenberg chain) on the full 2^N basis, its
 * ground state, the spin-current / energy-current / single-site operators applied to it, and the
 * dynamical correlation spectra S(omega).
 *
 * The reference has no library API: its seams are C++ member functions taking Eigen vectors.
 * Each entry point below names the reference function it replaces (file:line in the reference).
 *
 * Conventions
 *   - Basis order is the reference's: index k in [0, 2^N), bit s of k = site s, bit 0 = spin up
 *     (S^z = +1/2)  (src/QuantumBasis.h:36-60).
 *   - Vectors are interleaved complex: ESC_C128 = pairs of double, ESC_C64 = pairs of float.
 *   - Pointers are host memory unless ESC_DEVICE_PTR is set in `flags`, in which case they are
 *     device pointers on the handle's device.  Host pointers are copied in and out inside the
 *     call.  Calls on one handle are serial; each handle owns one CUDA stream and every call
 *     returns with that stream synchronised unless ESC_ASYNC is set (device pointers only).
 *   - Scalars (alpha, beta, E0, spectra) are always double.
 *   - No call throws; every call returns an esc_status and esc_last_error() explains failures.
 */
#ifndef ESC_H
#define ESC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    ESC_OK = 0,
    ESC_ERR_PARAM = 1,     /* bad or missing parameter (reference: std::invalid_argument) */
    ESC_ERR_MEMORY = 2,    /* device or host allocation failed / problem too large         */
    ESC_ERR_CUDA = 3,      /* CUDA runtime error                                           */
    ESC_ERR_NUMERIC = 4,   /* eigensolver failure, NaN in alpha/beta (reference: runtime_error) */
    ESC_ERR_STATE = 5,     /* call order (e.g. spectrum before a ground state)             */
    ESC_ERR_TIMEOUT = 6    /* a wait inside a kernel gave up (slab-pair H.v: the CTAs of one
                            * launch wait for each other's tiles, each wait at most ~1 s); the
                            * results of the calls since the last successful synchronisation are
                            * invalid, the handle stays usable.  Reported by the next call that
                            * synchronises the handle's stream. */
} esc_status;

typedef enum { ESC_C128 = 0, ESC_C64 = 1 } esc_dtype;

/* ESC_INTERNAL_ORDER: the vectors are in the handle's internal basis order (sites relabelled so
 * that the tiled H.v keeps bonds inside shared-memory tiles; see esc_basis_permutation).
 * Inner products and spectra do not depend on the order, so callers that keep vectors resident
 * can skip the permutation at the boundary. */
enum { ESC_DEVICE_PTR = 1, ESC_ASYNC = 2, ESC_INTERNAL_ORDER = 4 };

/* Operator identifiers for esc_apply_op (reference: Observables::ApplyOp, src/Observables.h:24-67,
 * plus the totals of :448-470, :664-699). */
typedef enum {
    ESC_OP_I = 0, ESC_OP_SX, ESC_OP_SY, ESC_OP_SZ, ESC_OP_SP, ESC_OP_SM, ESC_OP_SPE3, ESC_OP_SME3,
    ESC_OP_SXSYSZ, ESC_OP_JSX, ESC_OP_JSY, ESC_OP_JSZ, ESC_OP_JEX, ESC_OP_JEY, ESC_OP_JEXJEYJEZ,
    ESC_OP_JSXJSYJSZ, ESC_OP_JSX_TOTAL, ESC_OP_JSY_TOTAL, ESC_OP_JSZ_TOTAL, ESC_OP_JEX_TOTAL,
    ESC_OP_JEY_TOTAL, ESC_OP_JS_TOTAL, ESC_OP_JE_TOTAL, ESC_OP_COUNT
} esc_op;

/* Dynamics kinds (reference: StartDynamics dispatch, src/dynamics.h:43-60). */
typedef enum { ESC_DYN_JEJE = 0, ESC_DYN_JSJS = 1, ESC_DYN_LOCALSZSZ = 2 } esc_dyn_kind;

/* Spectrum method: Ritz = Lehmann sum over the ground-state Ritz pairs (the reference,
 * src/dynamics.h:277-307); CF = continued fraction from A|gs> (extension). */
typedef enum { ESC_DYNMODE_RITZ = 0, ESC_DYNMODE_CF = 1 } esc_dyn_mode;

typedef enum { ESC_START_REFUNIFORM = 0, ESC_START_NORMAL = 1 } esc_start_kind;

/* Parameter set.  Keys and defaults follow ConstVariables (src/ParametersEngine.h:21-149);
 * fields marked EXT are optional keys this library adds, with defaults equal to the reference's
 * hard-wired constants so that an unmodified reference input file gives the reference result. */
typedef struct {
    int Lx, Ly;                 /* NumberofSitesLx / NumberofSitesLy                          */
    int pbcx, pbcy;             /* IsPeriodicX / IsPeriodicY                                   */
    int seed;                   /* RandomSeed                                                  */
    char model[32];             /* Model: Kitaev | HeisenbergChain                             */
    char solver[16];            /* Solver: none (Lanczos) | ED                                 */
    char lanctype[16];          /* LancType: OnlyEgs | GS | All                                */
    double Kxx, Kyy, Kzz;
    double Bxx, Byy, Bzz;
    double temperature;         /* read, unused (as in the reference)                          */
    double lanczos_eps;         /* LanczosEps                                                  */
    int lanczos_steps;          /* LanczosSteps (default 200)                                  */
    int threads;                /* Threads (host threads for CPU-side work)                    */
    int local_skw;              /* LocalSkw -> spin-current dynamics (main.cpp:98-104)         */
    int spin_curr_dyn;          /* SpinCurrDynamics (read, unused by the reference main)       */
    int energy_curr_dyn;        /* EnergyCurrDynamics                                          */
    /* EXT */
    double jheis;               /* Jheis: Heisenberg J on every nearest-neighbour bond (0)     */
    int omega_steps;            /* OmegaSteps: omega = k*DOmega, k=0..OmegaSteps (1000)        */
    double domega;              /* DOmega (0.002)                                              */
    double eta;                 /* Eta (0.005)                                                 */
    int dyn_mode;               /* DynMode: Ritz | CF (Ritz)                                   */
    int dyn_lanczos_steps;      /* DynLanczosSteps for CF (LanczosSteps)                       */
    int precision;              /* Precision: fp64 | mixed (fp64)                              */
    int start_vector;           /* StartVector: RefUniform | Normal (RefUniform)               */
    int local_szsz_dyn;         /* LocalSzSzDynamics: run LocalDynSzSz from main (0)           */
    int reortho;                /* Reortho: 1 = full reorthogonalisation (reference), 0 = off  */
} esc_params;

/* Ground-state Lanczos configuration. */
typedef struct {
    int steps;                  /* MAXiter (LanczosSteps)                                      */
    double eps;                 /* LanczosEps                                                  */
    int lanctype;               /* 0 OnlyEgs, 1 GS, 2 All                                      */
    int reortho;                /* 1 = full Gram-Schmidt against every stored vector           */
    esc_dtype dtype;            /* storage/arithmetic of the Krylov vectors                    */
} esc_lanczos_cfg;

/* Dynamics configuration. */
typedef struct {
    int kind;                   /* esc_dyn_kind                                                */
    int mode;                   /* esc_dyn_mode                                                */
    int omega_steps;            /* rows = omega_steps + 1                                      */
    double domega, eta;
    int cf_steps;               /* continued-fraction Lanczos steps (CF mode)                  */
    esc_dtype dtype;            /* CF mode: precision of the CF Lanczos vectors                */
    int fp64_head;              /* CF mode, ESC_C64 only: leading CF steps run on complex128   *
                                 * vectors before the complex64 tail (0: 24 for JeJe, 48 for    *
                                 * the others; < 0: none)                                       */
} esc_dyn_cfg;

/* Batched continued-fraction Lanczos: ncols independent three-term recurrences (no
 * reorthogonalisation) from ncols start vectors, column c with its own field. */
typedef struct {
    int ncols;              /* 1..16                                                             */
    int max_steps;          /* recurrence steps per column (upper bound)                         */
    const int* steps;       /* per-column step limits (NULL: max_steps for every column)         */
    const double* fields;   /* ncols x 3 (Bxx, Byy, Bzz), NULL: the handle's field               */
    double tol;             /* a column stops when beta_k < tol * |phi|  (<= 0: 1e-10)           */
    esc_dtype dtype;        /* storage/arithmetic of the recurrence vectors                      */
    int use_graph;          /* 1: one iteration captured in a CUDA graph and replayed            */
    int fp64_head;          /* ESC_C64 only: the first fp64_head steps run on complex128 copies   *
                             * of the columns before the complex64 tail (0: none)                 */
} esc_cf_batch_cfg;

typedef struct esc_handle esc_handle;

/* ---- parameters -------------------------------------------------------------------------- */

/* Fill `p` with the reference defaults (LanczosSteps=200, Threads=1, omega grid 1001 x 0.002,
 * eta 0.005, Ritz mode, fp64, reference start vector). */
esc_status esc_params_default(esc_params* p);

/* Parse a reference input file.  Replaces ConstVariables::Initialize and its matchers
 * (src/ParametersEngine.h:53-149, :157-229): first line whose key matches exactly and whose
 * value parses wins; a missing mandatory key fails with "<Key>= argument is missing in the
 * input file!"; LocalSkw/SpinCurrDynamics/EnergyCurrDynamics require LancType=All. */
esc_status esc_params_from_file(const char* path, esc_params* p, char* errbuf, size_t errlen);

/* Neighbour table N x 3 (columns 0=z, 1=y, 2=x; -1 = none) of the cluster described by `p`,
 * computed on the host without a device.  Replaces Lattice::Honeycomb1 / Lattice::Chain
 * (src/Lattice.h:434-576, :60-136). */
esc_status esc_lattice(const esc_params* p, int* neigh, int* nsites);

/* Site relabelling and pass count of the tiled H.v for the model in `p` with tiles of 2^tile_bits
 * states whose lowest low_bits bits are shared (0 = default 3); host only.  tile_bits 0 = the
 * default of esc_create: 12, or 13 above 26 sites when that needs fewer passes.
 * bit_of_site (N entries, may be NULL), npasses (may be NULL).  No reference counterpart. */
esc_status esc_plan(const esc_params* p, int tile_bits, int low_bits, int* bit_of_site, int* npasses);

/* ---- handle --------------------------------------------------------------------------------- */

/* Build lattice, bond tables and device state.  Replaces the construction sequence
 * Lattice -> QBasis -> Hamiltonian(TightB_Ham, Diagonal) of main.cpp:56-73
 * (src/Lattice.h:37-58, src/QuantumBasis.h:36-46, src/Hamiltonian.h:44-54, :94-206, :331-377). */
esc_status esc_create(const esc_params* p, esc_handle** out);
esc_status esc_destroy(esc_handle* h);
const char* esc_last_error(const esc_handle* h);   /* h may be NULL: last error of this thread */

int esc_num_sites(const esc_handle* h);
int64_t esc_dim(const esc_handle* h);
/* Neighbour table N x 3 (columns 0=z, 1=y, 2=x; -1 = none), Lattice::N1neigh_
 * (src/Lattice.h:29, :497-564). */
esc_status esc_neighbors(const esc_handle* h, int* neigh);
/* bit_of_site[s] = position of site s's bit in the internal basis index (N entries). */
esc_status esc_basis_permutation(const esc_handle* h, int* bit_of_site);
/* The handle's CUDA stream (cudaStream_t), for callers that order their own work with it. */
void* esc_stream(esc_handle* h);

/* ---- operators -------------------------------------------------------------------------------- */

/* out = H in.  Replaces Hamiltonian::MatrixVectorMult (src/Hamiltonian.h:480-557); in != out. */
esc_status esc_hv(esc_handle* h, const void* in, void* out, esc_dtype dt, int flags);

/* OUT[:, c] = H(c) IN[:, c] for ncols columns stored with leading dimension ld (elements).
 * `fields` (ncols x 3 doubles: Bxx, Byy, Bzz per column) may be NULL to use the handle's field
 * for every column.  Batched form of MatrixVectorMult; no reference counterpart. */
esc_status esc_hv_batched(esc_handle* h, const void* in, void* out, int ncols, int64_t ld,
                          const double* fields, esc_dtype dt, int flags);

/* out = Op(site) in.  Replaces Observables::ApplyOp and the Apply* members
 * (src/Observables.h:24-67, :161-470, :488-607, :664-699).  `site` is ignored for totals. */
esc_status esc_apply_op(esc_handle* h, int op, int site, const void* in, void* out, esc_dtype dt,
                        int flags);

/* Reference start vector (src/DynLanczosSolver.h:57-59, :465-474) or the counter-based normal
 * start vector, normalised, in basis order. */
esc_status esc_start_vector(esc_handle* h, int kind, int seed, void* out, esc_dtype dt, int flags);

/* E = <v|H|v>/<v|v> evaluated in FP64 from a complex128 or complex64 vector, pass by pass without
 * forming H v (the FP64 refinement of a mixed-precision ground-state energy).  v == NULL: the
 * handle's last ground state in place (dt and flags ignored).  No reference counterpart. */
esc_status esc_rayleigh(esc_handle* h, const void* v, esc_dtype dt, int flags, double* E);

/* Allocation-free variant of esc_rayleigh, for callers that cannot allocate device memory: code
 * running inside another framework's memory pool or under a fixed memory budget, or a process
 * that must not grow its device footprint after start-up.  No counterpart in the reference.
 *   - No handle: the model comes from `p`; `v` is a DEVICE pointer to 2^N states in the
 *     reference basis order (complex128 or complex64 per `dt`); work is queued on `stream`
 *     (cudaStream_t, NULL = legacy default stream) and the call returns after synchronising it.
 *   - It calls no cudaMalloc/cudaFree and no allocating library routine.  Its scratch is a
 *     file-scope __device__ array of 2*8192 + 2*1216 + 8 doubles (about 150 KB) that every GPU
 *     which loads the library holds until the process exits.  The array holds one partial per
 *     tile of 2^12 states, so at most 25 sites (2^25 states) are accepted; larger models fail with
 *     ESC_ERR_PARAM and a message in esc_last_error(NULL).
 *   - The first call on a device (and the first after its context was rebuilt, e.g. by
 *     cudaDeviceReset) looks up the array's device address there, with that device current.
 *   - Every call synchronises `stream` and reads partial sums back to the host, so it must not be
 *     called while `stream` (or, in global capture mode, the legacy default stream) is being
 *     captured into a CUDA graph.
 *   - dt other than ESC_C128 / ESC_C64 fails with ESC_ERR_PARAM.
 *   - All calls share the one array: calls whose work overlaps on the GPU (other streams, other
 *     host threads, same device) race and may return wrong results.  Every value read back is
 *     written by the same call, so nothing has to be cleared between calls. */
esc_status esc_rayleigh_noalloc(const esc_params* p, const void* v, esc_dtype dt, void* stream, double* E);

/* FP64 residual refinement of the handle's ground state (extension; no reference counterpart),
 * for ground states from a complex64 Lanczos run.  Each of `steps` steps evaluates r = H psi - E psi
 * in FP64 (E = <psi|H|psi>, complex128 tiled passes) and replaces psi by the lowest Ritz vector of
 * H on span{psi, r}.  rnorm (may be NULL, steps+1 entries) receives |r| before each step and after
 * the last; E (may be NULL) the final <psi|H|psi>.  The refined vector becomes the handle's ground
 * state (complex128; esc_spectrum in CF mode starts from it; Ritz mode needs a new Lanczos run).
 * Needs two complex128 vectors of device memory. */
esc_status esc_refine_gs(esc_handle* h, int steps, double* E, double* rnorm);

/* ---- solvers ----------------------------------------------------------------------------------- */

/* Ground-state Lanczos.  Replaces DynLanczosSolver::Lanczos_Nirav (src/DynLanczosSolver.h:38-239)
 * including TriDiag (:371-414).  `start` (may be NULL: the handle's configured start vector) is
 * normalised by the call.  On return: alpha[0..steps-1], beta[0..steps] (beta[0] = 0), ritz
 * [0..steps-1] ascending, E0 = ritz[0]; gs_out (may be NULL) receives |gs> = PsiAll[0].
 * Arrays must hold cfg->steps (+1 for beta) entries.  The Krylov basis and the tridiagonal
 * eigenvectors stay in the handle for esc_spectrum (Ritz mode). */
esc_status esc_lanczos_gs(esc_handle* h, const esc_lanczos_cfg* cfg, const void* start, int flags,
                          double* E0, double* alpha, double* beta, double* ritz, int* steps,
                          void* gs_out);

/* Dense exact diagonalisation, the reference's Solver=ED.  Replaces ExactDiag +
 * DynLanczosSolver::fillFromED (src/Exactdiag.h:36-81, src/DynLanczosSolver.h:269-283, chosen in
 * main.cpp:79-83): the 2^N x 2^N complex128 matrix of H is built on the device and diagonalised
 * (cuSOLVER, loaded at run time); all 2^N eigenpairs then take the place of the Ritz pairs, so
 * esc_spectrum (Ritz mode) sums over the exact spectrum, and the ground state is the lowest
 * eigenvector.  evals (may be NULL): 2^N eigenvalues ascending; gs_out (may be NULL): the ground
 * state (host unless ESC_DEVICE_PTR).  At most 14 sites (the matrix is 4^N x 16 bytes). */
esc_status esc_exact_diag(esc_handle* h, double* evals, void* gs_out, int flags);

/* Batched continued-fraction coefficients (extension; the reference has no continued fraction).
 * starts: ncols vectors of 2^N states with stride ld (elements).  On return, for column c:
 * a[c*max_steps + k] (k < lens[c]) and b[c*(max_steps+1) + k] (k <= lens[c]), b[.. + 0] = |phi_c|,
 * so that <phi|(z-H)^-1|phi> = b0^2/(z - a0 - b1^2/(z - a1 - ...)). */
esc_status esc_cf_batched(esc_handle* h, const esc_cf_batch_cfg* cfg, const void* starts, int64_t ld, int flags,
                          double* a, double* b, int* lens);

/* Dynamical correlations of the last ground state.  Replaces DynJeJe / DynJsJs / LocalDynSzSz
 * (src/dynamics.h:345-460, :222-341, :64-217).  `out` receives (omega_steps+1) x ncols doubles in
 * the column order of the reference's JeJe_ (6) / JsJs_ (15) / 2SSLocal_ (9) files.  With
 * out == NULL only nrows / ncols are filled (nothing is computed). */
esc_status esc_spectrum(esc_handle* h, const esc_dyn_cfg* cfg, double* out, int* nrows, int* ncols);

/* Observables::TwoPointCorr (src/Observables.h:131-158): out (N x N complex, row-major) =
 * <gs| A_si B_sj |gs> for si >= sj, mirrored to (sj, si) without conjugation as the reference does.
 * opA / opB: single-site operators (ESC_OP_I .. ESC_OP_JSXJSYJSZ). */
esc_status esc_two_point(esc_handle* h, int opA, int opB, double* out);

/* Ground-state expectation values printed by Observables::measureLocalS / measureLocalJe
 * (src/Observables.h:107-128, :88-104): s_out N x 3 complex (<Sx>,<Sy>,<Sz>), je_out N x 2
 * complex (<Jex_i>,<Jey_i>).  Either may be NULL. */
esc_status esc_measure_local(esc_handle* h, double* s_out, double* je_out);

/* Self-tuning (extension, no reference counterpart): times the complex64 H.v of this Hamiltonian
 * on this device for each plan (tile bits 11/12/13, only 12/13 above 26 sites, x first-fit /
 * group-minimising term-to-pass assignment) and each kernel variant (ahead-of-time vs run-time
 * specialised, threads per tile, 2 or 3 tile buffers or staged epilogue loads) pass by pass,
 * composes the fastest variant of every pass and keeps the fastest composite.
 * All variants compute the same H.v.  Call before esc_lanczos_gs (it may change the internal
 * basis order; ESC_ERR_STATE otherwise).  Uses two complex64 vectors of scratch.  report (may be
 * NULL) receives one line per candidate and the choice.  ESC_AUTOTUNE=1 in the environment runs
 * it inside esc_create. */
esc_status esc_autotune(esc_handle* h, char* report, size_t report_len);

/* Gradients (extension, no reference counterpart).  dE0[3] = dE0/d{K, J, h} by
 * Hellmann-Feynman on the last ground state, with K the common Kitaev coupling
 * (Kxx=Kyy=Kzz=K) and h the [111] field (Bxx=Byy=Bzz=-h/sqrt3).  If dS is non-NULL it receives
 * (omega_steps+1) x 3 derivatives d Im S_tt(omega) / d{K,J,h} of the CF-mode total-current
 * spectrum of `kind`, by reverse mode through the continued fraction and the dynamical Lanczos
 * recurrence (vectors recomputed, not stored). */
esc_status esc_grad(esc_handle* h, const esc_dyn_cfg* cfg, double* dE0, double* dS);

/* ---- diagnostics ------------------------------------------------------------------------------- */

/* Arithmetic ceilings of the current device (no reference counterpart): out[0..2] = FP32 FMA,
 * packed f32x2 FMA and FP64 FMA throughput in TFLOP/s (an FMA counts 2 flops, a packed FMA 4),
 * out[3..5] = the timed kernels' durations in ms.  About three seconds of device time. */
esc_status esc_alu_peaks(double* out);

#ifdef __cplusplus
}
#endif
#endif /* ESC_H */
