// esc_abi.cpp -- the C ABI (include/esc.h): handle life cycle, staging of vectors across the
// boundary, H.v, operators, start vectors, and the entry points whose work lives in lanczos.cpp,
// spectra.cpp, grad.cpp and tune.cpp.
//
// Host C++ drives hand-written sm_103a kernels.  No CPU fallback exists: every vector operation
// runs on the device; the host only does O(M^2)-O(M^3) work on the tridiagonal matrix and the
// O(Omega x M) Lehmann / continued-fraction sums.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <type_traits>

#include "abi_common.h"

using esc::cplx;
using namespace escabi;

namespace {

thread_local std::string g_err;

}  // namespace

void esc::set_last_error(const std::string& msg) { g_err = msg; }

namespace escabi {

esc_status finish(esc_handle* h, esc_status st, const std::string& msg) {
    g_err = msg;
    if (h) h->err = msg;
    return st;
}

size_t esize(esc_dtype dt) { return dt == ESC_C64 ? 8 : 16; }
bool bad_dtype(int dt) { return dt != ESC_C128 && dt != ESC_C64; }

void ensure(void*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return;
    if (p) { cudaFree(p); p = nullptr; cap = 0; }
    if (need == 0) return;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        p = nullptr;
        throw Fail(ESC_ERR_MEMORY, "device allocation of " + std::to_string(need >> 20) + " MiB failed (" +
                                       cudaGetErrorString(e) + ")");
    }
    cap = need;
}
// Synchronises the handle's stream; reports a slab-pair wait that gave up since the last check
// (the flag is read only when slab-pair launches were made since then).
void sync(esc_handle* h) {
    ESC_CUDA(cudaStreamSynchronize(h->stream));
    if (!h->slab_sync) return;
    const unsigned long long n = esc::slab_pair_launches();
    if (n == h->slab_seen) return;
    h->slab_seen = n;
    unsigned e = 0;
    ESC_CUDA(cudaMemcpyAsync(&e, h->slab_sync, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    ESC_CUDA(cudaStreamSynchronize(h->stream));
    if (e) {
        ESC_CUDA(cudaMemsetAsync(h->slab_sync, 0, sizeof(unsigned), h->stream));
        ESC_CUDA(cudaStreamSynchronize(h->stream));
        throw Fail(ESC_ERR_TIMEOUT, "a slab-pair H.v launch gave up waiting for its tiles: the results since the last "
                                    "synchronisation are invalid");
    }
}

// Precomputed bond diagonal (the analogue of the reference's HDiag without the field term),
// 4 B/state for complex64, 8 B/state for complex128; computed on first use.  If it cannot be
// allocated the tiled kernel computes the diagonal itself (slower, same result).
const void* diag_for(esc_handle* h, esc_dtype dt) {
    const int i = dt == ESC_C64 ? 1 : 0;
    if (h->d_diag[i]) return h->d_diag[i];
    const size_t need = (size_t)h->D * (dt == ESC_C64 ? 4 : 8);
    if (cudaMalloc(&h->d_diag[i], need) != cudaSuccess) {
        (void)cudaGetLastError();
        h->d_diag[i] = nullptr;
        return nullptr;
    }
    h->diag_bytes[i] = need;
    if (dt == ESC_C64) esc::launch_diag<float>(h->dm, h->d_diag[i], h->D, h->stream);
    else esc::launch_diag<double>(h->dm, h->d_diag[i], h->D, h->stream);
    return h->d_diag[i];
}

void ensure_partials(esc_handle* h, int rows) {
    const size_t need = (size_t)std::max(rows, 4) * esc::RED_MAX_BLOCKS * 2 * sizeof(double);
    ensure_t(h->d_part, h->part_bytes, need);
}
int64_t part_cap_doubles(esc_handle* h) { return (int64_t)(h->part_bytes / sizeof(double)); }

void permute(esc_handle* h, const esc::DevPerm& p, const void* in, void* out, int64_t n, esc_dtype dt) {
    if (dt == ESC_C64) esc::launch_permute<float>(p, in, out, n, h->stream);
    else esc::launch_permute<double>(p, in, out, n, h->stream);
}

// Staged input/output.  The kernels work in the internal basis order; unless the caller says
// ESC_INTERNAL_ORDER, inputs are permuted in and outputs permuted out (through d_io), and host
// pointers are copied.  One call handles `cols` vectors of `n` elements with stride `ld`.
Staged stage(esc_handle* h, const void* in, void* out, int cols, int64_t ld, esc_dtype dt, int flags) {
    const size_t es = esize(dt);
    const int64_t n = h->D;
    const bool dev = flags & ESC_DEVICE_PTR, internal = flags & ESC_INTERNAL_ORDER;
    if (dev && internal) return {in, out, ld};
    const size_t vb = (size_t)n * es;
    ensure(h->d_io, h->io_bytes, 2 * (size_t)cols * vb);
    char* A = (char*)h->d_io;              // internal-order input
    char* B = A + (size_t)cols * vb;       // internal-order output / reference-order staging
    for (int c = 0; c < cols; c++) {
        if (!in) break;
        const char* src = (const char*)in + (size_t)c * ld * es;
        if (internal) {
            ESC_CUDA(cudaMemcpyAsync(A + c * vb, src, vb, cudaMemcpyHostToDevice, h->stream));
        } else if (dev) {
            permute(h, h->to_int, src, A + c * vb, n, dt);
        } else {
            ESC_CUDA(cudaMemcpyAsync(B + c * vb, src, vb, cudaMemcpyHostToDevice, h->stream));
            permute(h, h->to_int, B + c * vb, A + c * vb, n, dt);
        }
    }
    return {in ? A : nullptr, B, n};
}
// A staging buffer larger than `keep` bytes (the 6 vectors a pipelined host batch leaves) is
// released before a solver allocates its own vectors; cudaFree waits for work still using it.
void release_staging(esc_handle* h, size_t keep) {
    if (h->d_io && h->io_bytes > keep) {
        const cudaError_t e = cudaFree(h->d_io);
        h->d_io = nullptr;
        h->io_bytes = 0;
        ESC_CUDA(e);   // a failed free reports its own cause (often a sticky error of earlier work)
    }
}
void unstage(esc_handle* h, const Staged& s, void* out, int cols, int64_t ld, esc_dtype dt, int flags) {
    const size_t es = esize(dt);
    const int64_t n = h->D;
    const bool dev = flags & ESC_DEVICE_PTR, internal = flags & ESC_INTERNAL_ORDER;
    if (!(dev && internal) && out) {
        const size_t vb = (size_t)n * es;
        // staging for the reference-order / host copy (already there when stage() made it; a
        // result that lives elsewhere, e.g. the ground state, may need it allocated here)
        if (!internal && !dev) ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, (size_t)cols * vb));
        char* A = (char*)h->d_io;
        for (int c = 0; c < cols; c++) {
            char* dst = (char*)out + (size_t)c * ld * es;
            const char* res = (const char*)s.out + (size_t)c * vb;
            if (internal) {
                ESC_CUDA(cudaMemcpyAsync(dst, res, vb, cudaMemcpyDeviceToHost, h->stream));
            } else if (dev) {
                permute(h, h->to_ref, res, dst, n, dt);
            } else {
                permute(h, h->to_ref, res, A + c * vb, n, dt);
                ESC_CUDA(cudaMemcpyAsync(dst, A + c * vb, vb, cudaMemcpyDeviceToHost, h->stream));
            }
        }
    }
    if (!(flags & ESC_ASYNC) || !dev) sync(h);
}


esc::DevModel model_with_field(const esc_handle* h, double bx, double by, double bz) {
    esc::DevModel m = h->dm;
    m.fx = 0.5 * bx; m.fy = 0.5 * by; m.fz = 0.5 * bz;
    esc::fill_float_copies(m);
    return m;
}

}  // namespace escabi

// =============================================================================================
// C ABI
// =============================================================================================
namespace escabi {

std::vector<std::pair<int, int>> bond_pairs(const esc_handle* h) {
    std::vector<std::pair<int, int>> pairs;
    for (const auto& b : h->bonds)
        if (b.kx - b.ky != 0.0 || b.kx + b.ky != 0.0) pairs.push_back({b.i, b.j});
    return pairs;
}

// Installs a site relabelling + pass plan: relabelled model, passes, basis permutations.  The
// bond diagonal depends on the relabelling, so cached diagonal vectors are dropped.
void install_plan(esc_handle* h, const esc::Plan& plan, int balance, int stages, int tb_bits) {
    h->plan = plan;
    std::vector<esc::Bond> rb(h->bonds);
    for (auto& b : rb) { b.i = h->plan.perm[b.i]; b.j = h->plan.perm[b.j]; }
    h->dm = esc::make_dev_model(h->p, h->L, rb, h->p.Bxx, h->p.Byy, h->p.Bzz);
    h->dm.slab_sync = h->slab_sync;
    h->passes = esc::make_passes(h->plan, h->dm, balance, stages, tb_bits);
    std::vector<int> inv(h->N), fwd(h->N);
    for (int s = 0; s < h->N; s++) { inv[h->plan.perm[s]] = s; fwd[s] = h->plan.perm[s]; }
    h->to_int = esc::make_perm_table(inv);    // internal bit b reads reference bit inv[b]
    h->to_ref = esc::make_perm_table(fwd);    // reference bit s reads internal bit perm[s]
    for (int i = 0; i < 2; i++)
        if (h->d_diag[i]) {
            cudaFree(h->d_diag[i]);
            h->d_diag[i] = nullptr;
            h->diag_bytes[i] = 0;
        }
}

// Run-time specialised complex64 passes (hv_jit.cu): ESC_JIT=0 off, =1 on, =require on and an
// error if it fails; by default on from 2^22 states, where the compile time is repaid.
void specialise(esc_handle* h, std::vector<esc::DevPass>& passes, int force) {
    const char* je = std::getenv("ESC_JIT");
    bool jit = je ? std::strcmp(je, "0") != 0 : h->D >= (int64_t(1) << 22);
    if (force >= 0) jit = force == 1;
    if (!jit) return;
    std::string err;
    if (!esc::jit_compile(passes, err) && je && std::strcmp(je, "require") == 0)
        throw Fail(ESC_ERR_CUDA, "run-time specialisation of the H.v passes failed: " + err);
}

}  // namespace escabi

extern "C" {

const char* esc_last_error(const esc_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

esc_status esc_create(const esc_params* p, esc_handle** out) {
    if (!p || !out) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    *out = nullptr;
    std::unique_ptr<esc_handle> h(new esc_handle());
    esc_status st = guarded(h.get(), [&]() {
        h->p = *p;
        esc::build_lattice(*p, h->L);
        esc::build_bonds(*p, h->L, h->bonds);
        h->N = h->L.N;
        h->D = int64_t(1) << h->N;
        int T = 12, c = 3;
        const char* te = std::getenv("ESC_TILE_BITS");
        if (te) T = std::atoi(te);
        if (const char* e = std::getenv("ESC_TILE_LOW")) c = std::atoi(e);
        esc::Plan plan = esc::make_plan(h->N, bond_pairs(h.get()), T, c, 200);
        if (!te && h->N > 26) {
            // large bases: 8192-state tiles when they need fewer passes (N=32: 4 instead of 5)
            esc::Plan p13 = esc::make_plan(h->N, bond_pairs(h.get()), 13, c, 200);
            if (p13.tiles.size() < plan.tiles.size()) plan = p13;
        }
        install_plan(h.get(), plan, -1, 0);
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess || ndev == 0) {
            (void)cudaGetLastError();
            throw Fail(ESC_ERR_CUDA, "no CUDA device available: this library has no CPU path");
        }
        ESC_CUDA(cudaGetDevice(&h->device));
        ESC_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        ensure_partials(h.get(), 4);
        // slab-pair words (passes paired from SLAB_MIN_SITES sites, or at any size by ESC_SLAB_PAIRS=1)
        const int pe = esc::slab_pairs_env();
        if (pe == 1 || (pe < 0 && h->N >= esc::SLAB_MIN_SITES)) {
            const size_t bytes = esc::slab_sync_words(h->N) * sizeof(unsigned);
            ESC_CUDA(cudaMalloc((void**)&h->slab_sync, bytes));
            ESC_CUDA(cudaMemsetAsync(h->slab_sync, 0, bytes, h->stream));
            h->dm.slab_sync = h->slab_sync;
            h->slab_seen = esc::slab_pair_launches();
        }
        if (!load_tuning(h.get())) {
            specialise(h.get(), h->passes);
            if (const char* e = std::getenv("ESC_AUTOTUNE"))
                if (std::atoi(e) == 1) autotune(h.get(), nullptr);
        }
    });
    if (st != ESC_OK) {
        g_err = h->err;
        esc_destroy(h.release());
        return st;
    }
    *out = h.release();
    return ESC_OK;
}

esc_status esc_autotune(esc_handle* h, char* report, size_t report_len) {
    if (!h) return finish(h, ESC_ERR_PARAM, "null argument");
    return guarded(h, [&]() {
        const std::string r = autotune(h, nullptr);
        if (report && report_len) {
            const size_t n = std::min(report_len - 1, r.size());
            std::memcpy(report, r.data(), n);
            report[n] = 0;
        }
    });
}

esc_status esc_destroy(esc_handle* h) {
    if (!h) return ESC_OK;
    for (void* p : {(void*)h->d_part, (void*)h->d_sc, h->d_L, h->d_work, h->d_gs, h->d_io, h->d_diag[0], h->d_diag[1],
                    h->d_cfb, (void*)h->d_cfs, (void*)h->d_cfi, (void*)h->slab_sync})
        if (p) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    for (cudaStream_t x : {h->s_in, h->s_out})
        if (x) cudaStreamDestroy(x);
    for (int i = 0; i < 2; i++)
        for (cudaEvent_t e : {h->ev_in[i], h->ev_afree[i], h->ev_out[i], h->ev_outfree[i]})
            if (e) cudaEventDestroy(e);
    delete h;
    return ESC_OK;
}

int esc_num_sites(const esc_handle* h) { return h ? h->N : 0; }
int64_t esc_dim(const esc_handle* h) { return h ? h->D : 0; }
void* esc_stream(esc_handle* h) { return h ? (void*)h->stream : nullptr; }

esc_status esc_lattice(const esc_params* p, int* neigh, int* nsites) {
    if (!p) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    return guarded(nullptr, [&]() {
        esc::Lattice L;
        esc::build_lattice(*p, L);
        if (nsites) *nsites = L.N;
        if (neigh) std::memcpy(neigh, L.neigh.data(), L.neigh.size() * sizeof(int));
    });
}

esc_status esc_neighbors(const esc_handle* h, int* neigh) {
    if (!h || !neigh) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    std::memcpy(neigh, h->L.neigh.data(), h->L.neigh.size() * sizeof(int));
    return ESC_OK;
}

esc_status esc_basis_permutation(const esc_handle* h, int* bit_of_site) {
    if (!h || !bit_of_site) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    std::copy(h->plan.perm.begin(), h->plan.perm.end(), bit_of_site);
    return ESC_OK;
}

esc_status esc_hv(esc_handle* h, const void* in, void* out, esc_dtype dt, int flags) {
    if (!h || !in || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (in == out) return finish(h, ESC_ERR_PARAM, "esc_hv: in and out must differ");
    if (bad_dtype(dt)) return finish(h, ESC_ERR_PARAM, "esc_hv: dt must be ESC_C128 or ESC_C64");
    return guarded(h, [&]() {
        Staged s = stage(h, in, out, 1, h->D, dt, flags);
        const void* dg = diag_for(h, dt);
        if (dt == ESC_C64) esc::launch_hv_tiled<float>(h->dm, h->passes, s.in, s.out, h->D, dg, h->stream);
        else esc::launch_hv_tiled<double>(h->dm, h->passes, s.in, s.out, h->D, dg, h->stream);
        unstage(h, s, out, 1, h->D, dt, flags);
    });
}

}  // extern "C"

namespace escabi {

// Host-buffer batch, pipelined: column c's host->device copy (stream s_in), its H.v with the
// permutations (handle stream) and its device->host copy (stream s_out) overlap with the
// neighbouring columns' -- the host link is full duplex, so column c+1 comes in while column c-1
// goes out.  Two slots of three vectors: A (copy in), B (internal-order input, later the
// reference-order result), C (internal-order result).  Events keep a slot's buffers from being
// refilled before their last reader is done.  Returns false (nothing done) when the 6 vectors do
// not fit.
template <typename R>
bool hv_host_pipelined(esc_handle* h, const char* in, char* out, int ncols, int64_t ld, const double* fields,
                       esc_dtype dt, bool internal) {
    const int64_t D = h->D;
    const size_t es = esize(dt), vb = (size_t)D * es;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { (void)cudaGetLastError(); return false; }
    if (fr + h->io_bytes < 6 * vb + ((size_t)1 << 30)) return false;
    ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, 6 * vb));
    if (!h->s_in) ESC_CUDA(cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking));
    if (!h->s_out) ESC_CUDA(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
    for (int i = 0; i < 2; i++)
        for (cudaEvent_t* e : {&h->ev_in[i], &h->ev_afree[i], &h->ev_out[i], &h->ev_outfree[i]})
            if (!*e) ESC_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    const void* dg = diag_for(h, dt);
    // the copy streams start after the work already queued on the handle's stream
    ESC_CUDA(cudaEventRecord(h->ev_out[0], h->stream));
    ESC_CUDA(cudaStreamWaitEvent(h->s_in, h->ev_out[0], 0));
    ESC_CUDA(cudaStreamWaitEvent(h->s_out, h->ev_out[0], 0));
    for (int c = 0; c < ncols; c++) {
        const int s = c & 1;
        char* A = (char*)h->d_io + (size_t)(3 * s) * vb;
        char* B = A + vb;
        char* C = B + vb;
        const double* b = fields ? fields + 3 * c : nullptr;
        const esc::DevModel m = b ? model_with_field(h, b[0], b[1], b[2]) : h->dm;
        // copy in (slot's A free once column c-2 has read it)
        if (c >= 2) ESC_CUDA(cudaStreamWaitEvent(h->s_in, h->ev_afree[s], 0));
        ESC_CUDA(cudaMemcpyAsync(A, in + (size_t)c * ld * es, vb, cudaMemcpyHostToDevice, h->s_in));
        ESC_CUDA(cudaEventRecord(h->ev_in[s], h->s_in));
        // compute (slot's result buffer free once column c-2 has been copied out)
        ESC_CUDA(cudaStreamWaitEvent(h->stream, h->ev_in[s], 0));
        if (c >= 2) ESC_CUDA(cudaStreamWaitEvent(h->stream, h->ev_outfree[s], 0));
        const char* res;
        if (internal) {
            esc::launch_hv_tiled<R>(m, h->passes, A, C, D, dg, h->stream);
            ESC_CUDA(cudaEventRecord(h->ev_afree[s], h->stream));
            res = C;
        } else {
            permute(h, h->to_int, A, B, D, dt);
            ESC_CUDA(cudaEventRecord(h->ev_afree[s], h->stream));
            esc::launch_hv_tiled<R>(m, h->passes, B, C, D, dg, h->stream);
            permute(h, h->to_ref, C, B, D, dt);
            res = B;
        }
        ESC_CUDA(cudaEventRecord(h->ev_out[s], h->stream));
        // copy out
        ESC_CUDA(cudaStreamWaitEvent(h->s_out, h->ev_out[s], 0));
        ESC_CUDA(cudaMemcpyAsync(out + (size_t)c * ld * es, res, vb, cudaMemcpyDeviceToHost, h->s_out));
        ESC_CUDA(cudaEventRecord(h->ev_outfree[s], h->s_out));
    }
    ESC_CUDA(cudaStreamSynchronize(h->s_out));
    ESC_CUDA(cudaStreamSynchronize(h->s_in));
    sync(h);
    return true;
}

}  // namespace escabi

extern "C" {

esc_status esc_hv_batched(esc_handle* h, const void* in, void* out, int ncols, int64_t ld, const double* fields,
                          esc_dtype dt, int flags) {
    if (!h || !in || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (ncols < 1 || ncols > esc::MAX_COLS) return finish(h, ESC_ERR_PARAM, "ncols must be 1..16");
    if (ld < h->D) return finish(h, ESC_ERR_PARAM, "ld must be >= 2^N");
    if (bad_dtype(dt)) return finish(h, ESC_ERR_PARAM, "esc_hv_batched: dt must be ESC_C128 or ESC_C64");
    return guarded(h, [&]() {
        esc::DevFields f;
        for (int c = 0; c < esc::MAX_COLS; c++) {
            const double* b = (fields && c < ncols) ? fields + 3 * c : nullptr;
            f.fx[c] = 0.5 * (b ? b[0] : h->p.Bxx);
            f.fy[c] = 0.5 * (b ? b[1] : h->p.Byy);
            f.fz[c] = 0.5 * (b ? b[2] : h->p.Bzz);
            f.fxf[c] = (float)f.fx[c]; f.fyf[c] = (float)f.fy[c]; f.fzf[c] = (float)f.fz[c];
        }
        if (!(flags & ESC_DEVICE_PTR) && ncols >= 2) {
            const bool internal = flags & ESC_INTERNAL_ORDER;
            const bool done = dt == ESC_C64
                                  ? hv_host_pipelined<float>(h, (const char*)in, (char*)out, ncols, ld, fields, dt, internal)
                                  : hv_host_pipelined<double>(h, (const char*)in, (char*)out, ncols, ld, fields, dt, internal);
            if (done) return;
        }
        // device pointers (or a host batch that did not fit the pipeline): the tiled passes over
        // all columns at once (tile offsets and term groups decoded once per tile for every column)
        Staged s = stage(h, in, out, ncols, ld, dt, flags);
        esc::DevCols cols = esc::single_column(h->dm);
        cols.ncols = ncols;
        cols.ld = s.ld;
        cols.f = f;
        const void* dg = diag_for(h, dt);
        if (dt == ESC_C64) esc::launch_hv_cols<float>(h->dm, cols, h->passes, s.in, s.out, h->D, dg, h->stream, nullptr);
        else esc::launch_hv_cols<double>(h->dm, cols, h->passes, s.in, s.out, h->D, dg, h->stream, nullptr);
        unstage(h, s, out, ncols, ld, dt, flags);
    });
}

esc_status esc_apply_op(esc_handle* h, int op, int site, const void* in, void* out, esc_dtype dt, int flags) {
    if (!h || !in || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (in == out) return finish(h, ESC_ERR_PARAM, "esc_apply_op: in and out must differ");
    if (bad_dtype(dt)) return finish(h, ESC_ERR_PARAM, "esc_apply_op: dt must be ESC_C128 or ESC_C64");
    return guarded(h, [&]() {
        const esc::DevOp d = esc::make_dev_op(esc::operator_terms(op, site, h->p, h->L), &h->plan.perm);
        Staged s = stage(h, in, out, 1, h->D, dt, flags);
        if (dt == ESC_C64) esc::launch_apply<float>(d, s.in, s.out, h->D, h->stream);
        else esc::launch_apply<double>(d, s.in, s.out, h->D, h->stream);
        unstage(h, s, out, 1, h->D, dt, flags);
    });
}

// Start vector into `dst` (device, internal order, normalised).  Generated in the reference basis
// order (the reference's draw order) and permuted; uses d_work as scratch.
}  // extern "C"

namespace escabi {

void start_vector_internal(esc_handle* h, int kind, int seed, void* dst, esc_dtype dt) {
    const int64_t D = h->D;
    // generation buffer: complex128 staging only for the host-generated reference start vector
    const size_t gbytes = (size_t)D * (kind == ESC_START_REFUNIFORM ? 16 : esize(dt));
    ensure(h->d_work, h->work_bytes, std::max(h->work_bytes, gbytes));
    ensure_t(h->d_sc, h->sc_bytes, std::max<size_t>(h->sc_bytes, 64));
    void* gen = h->d_work;
    if (kind == ESC_START_REFUNIFORM) {
        std::vector<cplx> v((size_t)D);
        esc::ref_uniform_start(seed, D, v.data());
        ESC_CUDA(cudaMemcpyAsync(gen, v.data(), (size_t)D * 16, cudaMemcpyHostToDevice, h->stream));
        if (dt == ESC_C64) {
            esc::launch_convert_c128_to_c64(gen, dst, D, h->stream);
            ESC_CUDA(cudaMemcpyAsync(gen, dst, (size_t)D * 8, cudaMemcpyDeviceToDevice, h->stream));
        }
        sync(h);
    } else if (kind == ESC_START_NORMAL) {
        if (dt == ESC_C128) esc::launch_start_normal<double>((uint64_t)(int64_t)seed, gen, D, h->stream);
        else esc::launch_start_normal<float>((uint64_t)(int64_t)seed, gen, D, h->stream);
    } else {
        throw Fail(ESC_ERR_PARAM, "unknown start-vector kind");
    }
    permute(h, h->to_int, gen, dst, D, dt);
    if (dt == ESC_C128) { esc::launch_nrm2<double>(dst, D, h->d_part, h->d_sc, h->stream); esc::launch_scale_rsqrt<double>(dst, dst, h->d_sc, D, h->stream); }
    else { esc::launch_nrm2<float>(dst, D, h->d_part, h->d_sc, h->stream); esc::launch_scale_rsqrt<float>(dst, dst, h->d_sc, D, h->stream); }
}

}  // namespace escabi

extern "C" {

esc_status esc_start_vector(esc_handle* h, int kind, int seed, void* out, esc_dtype dt, int flags) {
    if (!h || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (bad_dtype(dt)) return finish(h, ESC_ERR_PARAM, "esc_start_vector: dt must be ESC_C128 or ESC_C64");
    return guarded(h, [&]() {
        Staged s = stage(h, nullptr, out, 1, h->D, dt, flags);
        start_vector_internal(h, kind, seed, s.out, dt);
        unstage(h, s, out, 1, h->D, dt, flags);
    });
}

esc_status esc_lanczos_gs(esc_handle* h, const esc_lanczos_cfg* cfg, const void* start, int flags, double* E0,
                          double* alpha, double* beta, double* ritz, int* steps, void* gs_out) {
    if (!h || !cfg) return finish(h, ESC_ERR_PARAM, "null argument");
    if (cfg->steps < 2) return finish(h, ESC_ERR_PARAM, "LanczosSteps must be >= 2");
    if (cfg->lanctype < 0 || cfg->lanctype > 2) return finish(h, ESC_ERR_PARAM, "DynLanczosSolver: Use PsiOrAll==GS or All");
    if (bad_dtype(cfg->dtype)) return finish(h, ESC_ERR_PARAM, "esc_lanczos_gs: dtype must be ESC_C128 or ESC_C64");
    return guarded(h, [&]() {
        const int64_t D = h->D;
        const esc_dtype dt = cfg->dtype;
        release_staging(h, 2 * (size_t)D * esize(dt));
        // start vector -> internal order in d_io[0]
        Staged s = stage(h, start, nullptr, 1, D, dt, flags);
        void* d_start = (void*)s.in;
        if (!start) {
            ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, (size_t)D * esize(dt)));
            d_start = h->d_io;
            start_vector_internal(h, h->p.start_vector, h->p.seed, d_start, dt);
        }
        if (dt == ESC_C64) lanczos_gs<float>(h, *cfg, d_start);
        else lanczos_gs<double>(h, *cfg, d_start);
        const int n = h->nsteps;
        if (steps) *steps = n;
        if (E0) *E0 = h->ritz[0];
        if (alpha) std::copy(h->alpha.begin(), h->alpha.end(), alpha);
        if (beta) std::copy(h->beta.begin(), h->beta.end(), beta);
        if (ritz) std::copy(h->ritz.begin(), h->ritz.end(), ritz);
        if (gs_out) {
            Staged g{nullptr, h->d_gs, D};
            unstage(h, g, gs_out, 1, D, dt, flags & ~ESC_ASYNC);
        }
        sync(h);
        if (h->d_io) {   // start vector and export staging are no longer needed: room for the dynamics
            cudaFree(h->d_io);
            h->d_io = nullptr;
            h->io_bytes = 0;
        }
    });
}

}  // extern "C"

extern "C" {

esc_status esc_spectrum(esc_handle* h, const esc_dyn_cfg* cfg, double* out, int* nrows, int* ncols) {
    if (!h || !cfg) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    if (cfg->mode == ESC_DYNMODE_RITZ && !h->have_basis)
        return finish(h, ESC_ERR_STATE, "You need to set LancType=All for Dynamical calculations --- you dummy!");
    if (cfg->omega_steps < 0) return finish(h, ESC_ERR_PARAM, "omega_steps must be >= 0");
    if (!out) {   // size query: nothing is computed
        const int nc = cfg->kind == ESC_DYN_JEJE ? 6 : cfg->kind == ESC_DYN_JSJS ? 15 : cfg->kind == ESC_DYN_LOCALSZSZ ? 9 : 0;
        if (!nc) return finish(h, ESC_ERR_PARAM, "Unknown dynstr parameter");
        if (nrows) *nrows = cfg->omega_steps + 1;
        if (ncols) *ncols = nc;
        return finish(h, ESC_OK, "");
    }
    return guarded(h, [&]() {
        release_staging(h, 0);   // the spectra stage nothing through it
        std::vector<double> s;
        int nc = 0;
        // Ritz mode runs in the precision of the ground state and its Krylov basis.  CF mode runs
        // in complex64 when either the ground state or cfg->dtype is complex64; a complex128
        // ground state is then rounded once to complex64 for the duration of the call.
        const esc_dtype dt = h->basis_dt;
        if (dt == ESC_C64) {
            spectrum_impl<float>(h, *cfg, s, nc);
        } else if (cfg->mode == ESC_DYNMODE_CF && cfg->dtype == ESC_C64) {
            void* g32 = nullptr;
            ESC_CUDA(cudaMalloc(&g32, (size_t)h->D * 8));
            esc::launch_convert_c128_to_c64(h->d_gs, g32, h->D, h->stream);
            void* g64 = h->d_gs;
            h->d_gs = g32;
            try {
                spectrum_impl<float>(h, *cfg, s, nc);
            } catch (...) {
                h->d_gs = g64;
                (void)cudaStreamSynchronize(h->stream);
                cudaFree(g32);
                throw;
            }
            h->d_gs = g64;
            sync(h);
            cudaFree(g32);
        } else {
            spectrum_impl<double>(h, *cfg, s, nc);
        }
        if (nrows) *nrows = cfg->omega_steps + 1;
        if (ncols) *ncols = nc;
        if (out) std::copy(s.begin(), s.end(), out);
    });
}

esc_status esc_two_point(esc_handle* h, int opA, int opB, double* out) {
    if (!h || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    for (int op : {opA, opB})
        if (op < 0 || op > ESC_OP_JSXJSYJSZ) return finish(h, ESC_ERR_PARAM, "Unknown Operator label");
    return guarded(h, [&]() {
        std::vector<cplx> C;
        if (h->basis_dt == ESC_C64) two_point_impl<float>(h, opA, opB, C);
        else two_point_impl<double>(h, opA, opB, C);
        std::memcpy(out, C.data(), C.size() * sizeof(cplx));
    });
}

esc_status esc_measure_local(esc_handle* h, double* s_out, double* je_out) {
    if (!h) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    return guarded(h, [&]() {
        auto run = [&](auto tag) {
            typedef decltype(tag) R;
            Spectra<R> S(h);
            ensure(h->d_work, h->work_bytes, std::max(h->work_bytes, (size_t)h->D * Pipe<R>::ES));
            ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)16 * sizeof(double)));
            double* d_tmp = h->d_sc;
            for (int s = 0; s < h->N; s++) {
                if (s_out) {
                    const int ops[3] = {ESC_OP_SX, ESC_OP_SY, ESC_OP_SZ};
                    for (int c = 0; c < 3; c++) {
                        const cplx v = S.expect(esc::operator_terms(ops[c], s, h->p, h->L), 0, d_tmp);
                        s_out[(s * 3 + c) * 2] = v.real(); s_out[(s * 3 + c) * 2 + 1] = v.imag();
                    }
                }
                if (je_out) {
                    const int ops[2] = {ESC_OP_JEX, ESC_OP_JEY};
                    for (int c = 0; c < 2; c++) {
                        const cplx v = S.expect(esc::operator_terms(ops[c], s, h->p, h->L), 0, d_tmp);
                        je_out[(s * 2 + c) * 2] = v.real(); je_out[(s * 2 + c) * 2 + 1] = v.imag();
                    }
                }
            }
        };
        if (h->basis_dt == ESC_C64) run(float()); else run(double());
    });
}

esc_status esc_grad(esc_handle* h, const esc_dyn_cfg* cfg, double* dE0, double* dS) {
    if (!h || !dE0) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    if (dS && !cfg) return finish(h, ESC_ERR_PARAM, "dS needs a dynamics configuration");
    if (dS && h->basis_dt != ESC_C128) return finish(h, ESC_ERR_STATE, "dS(omega) gradients run in FP64: compute the ground state with ESC_C128");
    return guarded(h, [&]() { grad_impl(h, cfg, dE0, dS); });
}

}  // extern "C"

extern "C" esc_status esc_plan(const esc_params* p, int tile_bits, int low_bits, int* bit_of_site, int* npasses) {
    if (!p) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    return guarded(nullptr, [&]() {
        esc::Lattice L;
        std::vector<esc::Bond> bonds;
        esc::build_lattice(*p, L);
        esc::build_bonds(*p, L, bonds);
        std::vector<std::pair<int, int>> pairs;
        for (const auto& b : bonds)
            if (b.kx - b.ky != 0.0 || b.kx + b.ky != 0.0) pairs.push_back({b.i, b.j});
        const int c = low_bits > 0 ? low_bits : 3;
        esc::Plan P = esc::make_plan(L.N, pairs, tile_bits > 0 ? tile_bits : 12, c, 200);
        if (tile_bits <= 0 && L.N > 26) {   // the default of esc_create
            esc::Plan p13 = esc::make_plan(L.N, pairs, 13, c, 200);
            if (p13.tiles.size() < P.tiles.size()) P = p13;
        }
        std::vector<esc::Bond> rb(bonds);
        for (auto& b : rb) { b.i = P.perm[b.i]; b.j = P.perm[b.j]; }
        const esc::DevModel m = esc::make_dev_model(*p, L, rb, p->Bxx, p->Byy, p->Bzz);
        const auto passes = esc::make_passes(P, m);   // throws if a term fits no tile
        if (bit_of_site) std::copy(P.perm.begin(), P.perm.end(), bit_of_site);
        if (npasses) *npasses = (int)passes.size();
    });
}

extern "C" esc_status esc_rayleigh(esc_handle* h, const void* v, esc_dtype dt, int flags, double* E) {
    if (!h || !E) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!v && !h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    if (v && bad_dtype(dt)) return finish(h, ESC_ERR_PARAM, "esc_rayleigh: dt must be ESC_C128 or ESC_C64");
    return guarded(h, [&]() {
        // v == NULL: the handle's ground state, in place (no copy of the vector)
        if (!v) {
            dt = h->basis_dt;
            flags = ESC_DEVICE_PTR | ESC_INTERNAL_ORDER;
        }
        Staged s = stage(h, v ? v : h->d_gs, nullptr, 1, h->D, dt, flags);
        ensure_partials(h, 4);
        std::vector<double> num;
        const int maxb = esc::RED_MAX_BLOCKS;
        if (dt == ESC_C64) esc::launch_energy<float>(h->dm, h->passes, s.in, h->D, h->d_part, maxb, num, h->stream);
        else esc::launch_energy<double>(h->dm, h->passes, s.in, h->D, h->d_part, maxb, num, h->stream);
        ensure_t(h->d_sc, h->sc_bytes, std::max<size_t>(h->sc_bytes, 64));
        if (dt == ESC_C64) esc::launch_dot<float>(s.in, s.in, h->D, h->d_part, h->d_sc, h->stream);
        else esc::launch_dot<double>(s.in, s.in, h->D, h->d_part, h->d_sc, h->stream);
        double nn[2];
        ESC_CUDA(cudaMemcpyAsync(nn, h->d_sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        sync(h);
        *E = num[0] / nn[0];
    });
}

extern "C" esc_status esc_refine_gs(esc_handle* h, int steps, double* E, double* rnorm) {
    if (!h) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    if (steps < 0) return finish(h, ESC_ERR_PARAM, "steps must be >= 0");
    return guarded(h, [&]() { refine_gs(h, steps, E, rnorm); });
}

extern "C" esc_status esc_cf_batched(esc_handle* h, const esc_cf_batch_cfg* cfg, const void* starts, int64_t ld,
                                     int flags, double* a, double* b, int* lens) {
    if (!h || !cfg || !starts) return finish(h, ESC_ERR_PARAM, "null argument");
    if (cfg->ncols < 1 || cfg->ncols > esc::MAX_COLS) return finish(h, ESC_ERR_PARAM, "ncols must be 1..16");
    if (cfg->max_steps < 1) return finish(h, ESC_ERR_PARAM, "max_steps must be >= 1");
    if (bad_dtype(cfg->dtype)) return finish(h, ESC_ERR_PARAM, "esc_cf_batched: dtype must be ESC_C128 or ESC_C64");
    if (ld < h->D) return finish(h, ESC_ERR_PARAM, "ld must be >= 2^N");
    return guarded(h, [&]() {
        const int nc = cfg->ncols, K = cfg->max_steps;
        const esc_dtype dt = cfg->dtype;
        const size_t es = esize(dt), vb = (size_t)h->D * es;
        release_staging(h, vb);
        ensure(h->d_cfb, h->cfb_bytes, std::max(h->cfb_bytes, 3 * (size_t)nc * vb));
        char* set1 = (char*)h->d_cfb + (size_t)nc * vb;
        for (int c = 0; c < nc; c++) {
            const char* src = (const char*)starts + (size_t)c * ld * es;
            const bool dev = flags & ESC_DEVICE_PTR, internal = flags & ESC_INTERNAL_ORDER;
            if (internal) {
                ESC_CUDA(cudaMemcpyAsync(set1 + c * vb, src, vb, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
            } else if (dev) {
                permute(h, h->to_int, src, set1 + c * vb, h->D, dt);
            } else {
                ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, vb));
                ESC_CUDA(cudaMemcpyAsync(h->d_io, src, vb, cudaMemcpyHostToDevice, h->stream));
                permute(h, h->to_int, h->d_io, set1 + c * vb, h->D, dt);
            }
        }
        std::vector<int> steps(nc, K);
        if (cfg->steps)
            for (int c = 0; c < nc; c++) steps[c] = std::max(1, std::min(K, cfg->steps[c]));
        std::vector<esc::DevModel> ms(nc, h->dm);
        if (cfg->fields)
            for (int c = 0; c < nc; c++) ms[c] = model_with_field(h, cfg->fields[3 * c], cfg->fields[3 * c + 1], cfg->fields[3 * c + 2]);
        const double tol = cfg->tol > 0 ? cfg->tol : 1e-10;
        std::vector<std::vector<double>> A, B;
        if (dt == ESC_C64) cf_batch_run<float>(h, nc, K, steps, ms, tol, cfg->use_graph != 0, A, B, std::max(0, cfg->fp64_head));
        else cf_batch_run<double>(h, nc, K, steps, ms, tol, cfg->use_graph != 0, A, B);
        for (int c = 0; c < nc; c++) {
            if (lens) lens[c] = (int)A[c].size();
            if (a) for (size_t k = 0; k < A[c].size(); k++) a[(size_t)c * K + k] = A[c][k];
            if (b) for (size_t k = 0; k < B[c].size(); k++) b[(size_t)c * (K + 1) + k] = B[c][k];
        }
    });
}
