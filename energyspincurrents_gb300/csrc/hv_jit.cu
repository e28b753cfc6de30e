// hv_jit.cu -- run-time specialisation of the complex64 H.v passes.
//
// The term groups of a pass (which thread-bit mask, which register mask, which coupling) are
// fixed once the Hamiltonian and the plan are known.  The ahead-of-time kernel reads them from the
// pass table and dispatches on them per term; here they are written out as straight-line code
// around the same pass body (hv_pass_device.cuh), compiled with NVRTC for the current device and
// loaded with the driver API.  The generated kernel performs the same floating-point operations in
// the same order as the ahead-of-time kernel, so the two give identical results.
//
// Modules are cached per (device, source) for the life of the process.
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "esc_internal.h"
#include "hv_pass_device.cuh"

namespace esc {

namespace {

const char* kPassDeviceSource =
#include "hv_pass_device.inc"
    ;

struct JitEntry {
    int device;
    CUfunction fn;
    int E, TB;
    int per_sm;
    size_t smem;
};

std::mutex g_mu;
std::vector<JitEntry> g_entries;
std::map<std::string, std::vector<int>> g_cache;   // device + source -> entry per kernel

// 4096-state tiles (and 2048): 512, 256 or 128 threads; 8192-state tiles: 1024, 512 or 256 threads
bool eligible(const DevPass& p) {
    const bool shape = (p.Tp == 11 || p.Tp == 12) ? p.tb_bits >= 7 && p.tb_bits <= 9 : p.Tp == 13 && p.tb_bits >= 8 && p.tb_bits <= 10;
    return p.c == 3 && shape && p.nterm > 0;
}

// CTAs per SM of the register budget: two for 4096-state tiles, one for 8192 (2 x 64 KB ring)
int min_ctas(const DevPass& p) { return p.Tp >= 13 ? 1 : 2; }

std::string hexf(float x) {
    unsigned u;
    std::memcpy(&u, &x, 4);
    char b[32];
    std::snprintf(b, sizeof b, "__int_as_float(0x%08xu)", u);
    return b;
}

// Straight-line terms functor of one pass: the group loop of RuntimeTerms (hv_tiled.cu) unrolled.
std::string terms_source(const DevPass& p, int k) {
    const int TB = 1 << p.tb_bits;
    const int E = 1 << (p.Tp - p.tb_bits);
    std::ostringstream o;
    o << "struct Terms" << k << " {\n"
      << "  __device__ __forceinline__ void operator()(const float2* tile, int tid, float2 vfx, float fy, float2 (&acc)["
      << E << "]) const {\n";
    int q = 0;
    for (int g = 0; g < p.ngroup; g++) {
        o << "    {\n      const unsigned glo = " << p.glo[g] << "u;\n      float2 P[" << E << "];\n"
          << "      escdev::load_group<" << E << ", " << TB << ">(tile, tid, glo, P);\n"
          << "      const bool par = __popc((unsigned)tid & glo) & 1; (void)par;\n"
          << "      const float sf = ((unsigned)tid & glo) ? fy : -fy; (void)sf;\n";
        for (int n = 0; n < p.gnt[g]; n++, q++) {
            const int code = p.gk[q];
            if (code < 32) {
                o << "      { const float a = " << hexf(p.ga[q]) << ", b = " << hexf(p.gb[q]) << ";\n"
                  << "        const float2 vA = par ? make_float2(b, b) : make_float2(a, a);\n"
                  << "        const float2 vB = par ? make_float2(a, a) : make_float2(b, b);\n"
                  << "        escdev::gbond<" << E << ", " << code << ">(P, vA, vB, acc); }\n";
            } else {
                o << "      escdev::gfield<" << E << ", " << (code - 33) << ">(P, vfx, fy, sf, acc);\n";
            }
        }
        o << "    }\n";
    }
    o << "  }\n};\n"
      << "extern \"C\" __global__ void __launch_bounds__(" << TB << ", " << min_ctas(p) << ") esc_jit_pass" << k
      << "(const __grid_constant__ escdev::PassTab p, const float* __restrict__ diag, const float2* __restrict__ in,"
         " float2* __restrict__ out, long long ntiles, const int* __restrict__ active) {\n"
      << "  escdev::pass_body<" << E << ", " << (p.stages >= 2 && p.stages <= 5 ? p.stages : 2) << ", Terms" << k << ", "
      << TB << ">(p, Terms" << k << "{}, diag, in, out, ntiles, active);\n}\n";
    return o.str();
}

// Slab-pair kernel q of passes a, b (terms functors Terms<ka>, Terms<kb>): pair_body of
// hv_pass_device.cuh, launched cooperatively.
std::string pair_source(const DevPass& a, int ka, int kb, int q) {
    const int TB = 1 << a.tb_bits;
    const int E = 1 << (a.Tp - a.tb_bits);
    std::ostringstream o;
    o << "extern \"C\" __global__ void __launch_bounds__(" << TB << ", " << min_ctas(a) << ") esc_jit_pair" << q
      << "(const __grid_constant__ escdev::PassTab pa, const __grid_constant__ escdev::PassTab pb,"
         " const __grid_constant__ escdev::PairTab st, const float* __restrict__ diag, const float2* __restrict__ in,"
         " float2* __restrict__ out, const int* __restrict__ active) {\n"
      << "  escdev::pair_body<" << E << ", " << TB << ">(pa, pb, st, Terms" << ka << "{}, Terms" << kb
      << "{}, diag, in, out, active);\n}\n";
    return o.str();
}

// Driver entry points, resolved through the runtime (the library links no libcuda, so that it
// also loads on hosts without a GPU driver).
struct Driver {
    decltype(&::cuModuleLoadData) moduleLoadData = nullptr;
    decltype(&::cuModuleGetFunction) moduleGetFunction = nullptr;
    decltype(&::cuFuncSetAttribute) funcSetAttribute = nullptr;
    decltype(&::cuOccupancyMaxActiveBlocksPerMultiprocessor) occupancy = nullptr;
    decltype(&::cuLaunchKernel) launchKernel = nullptr;
    decltype(&::cuLaunchCooperativeKernel) launchCooperative = nullptr;
    decltype(&::cuGetErrorString) getErrorString = nullptr;
    bool ok = false;
};

template <typename F>
bool resolve(const char* name, F& f) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
        (void)cudaGetLastError();
        return false;
    }
    f = reinterpret_cast<F>(p);
    return true;
}

const Driver& driver() {
    static Driver d = [] {
        Driver x;
        x.ok = resolve("cuModuleLoadData", x.moduleLoadData) && resolve("cuModuleGetFunction", x.moduleGetFunction) &&
               resolve("cuFuncSetAttribute", x.funcSetAttribute) &&
               resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", x.occupancy) &&
               resolve("cuLaunchKernel", x.launchKernel) && resolve("cuGetErrorString", x.getErrorString) &&
               resolve("cuLaunchCooperativeKernel", x.launchCooperative);
        return x;
    }();
    return d;
}

bool drv(CUresult r, const char* what, std::string& err) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    if (driver().getErrorString) driver().getErrorString(r, &s);
    err = std::string(what) + ": " + (s ? s : "unknown driver error");
    return false;
}

}  // namespace

std::string jit_source(const std::vector<DevPass>& passes, std::vector<int>* which, std::vector<int>* pairs) {
    std::string src(kPassDeviceSource);
    std::vector<int> kof(passes.size(), -1);
    int k = 0;
    for (size_t i = 0; i < passes.size(); i++)
        if (eligible(passes[i])) {
            src += terms_source(passes[i], k);
            kof[i] = k++;
            if (which) which->push_back((int)i);
        }
    // slab pairs of two specialised passes of one shape
    int q = 0;
    for (size_t i = 0; i + 1 < passes.size(); i++) {
        const DevPass& a = passes[i];
        const DevPass& b = passes[i + 1];
        if (a.pair && kof[i] >= 0 && kof[i + 1] >= 0 && a.tb_bits == b.tb_bits && a.Tp == b.Tp) {
            src += pair_source(a, kof[i], kof[i + 1], q++);
            if (pairs) pairs->push_back((int)i);
        }
    }
    return src;
}

bool jit_compile(std::vector<DevPass>& passes, std::string& err) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaFree(0) != cudaSuccess) {
        (void)cudaGetLastError();
        err = "no CUDA context";
        return false;
    }
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    std::vector<int> which, pairs;
    const std::string src = jit_source(passes, &which, &pairs);
    if (which.empty()) return true;
    const Driver& D = driver();
    if (!D.ok) {
        err = "driver entry points unavailable";
        return false;
    }
    const std::string arch = "-arch=sm_" + std::to_string(major * 10 + minor) + "a";
    const std::string key = std::to_string(dev) + arch + src;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it == g_cache.end()) {
        nvrtcProgram prog;
        if (nvrtcCreateProgram(&prog, src.c_str(), "esc_hv_pass.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
            err = "nvrtcCreateProgram failed";
            return false;
        }
        const char* opts[] = {arch.c_str(), "-std=c++17"};
        const nvrtcResult rc = nvrtcCompileProgram(prog, 2, opts);
        if (rc != NVRTC_SUCCESS) {
            size_t n = 0;
            nvrtcGetProgramLogSize(prog, &n);
            std::string log(n, '\0');
            nvrtcGetProgramLog(prog, &log[0]);
            nvrtcDestroyProgram(&prog);
            err = std::string("NVRTC: ") + nvrtcGetErrorString(rc) + "\n" + log;
            return false;
        }
        size_t n = 0;
        nvrtcGetCUBINSize(prog, &n);
        std::vector<char> cubin(n);
        nvrtcGetCUBIN(prog, cubin.data());
        nvrtcDestroyProgram(&prog);
        CUmodule mod;
        if (!drv(D.moduleLoadData(&mod, cubin.data()), "cuModuleLoadData", err)) return false;
        std::vector<int> ids;
        for (size_t k = 0; k < which.size(); k++) {
            const DevPass& p = passes[which[k]];
            JitEntry e;
            e.device = dev;
            e.TB = 1 << p.tb_bits;
            e.E = 1 << (p.Tp - p.tb_bits);
            e.smem = (size_t)(p.stages >= 3 ? 3 : 2) * e.TB * e.E * sizeof(float2);
            const std::string name = "esc_jit_pass" + std::to_string(k);
            if (!drv(D.moduleGetFunction(&e.fn, mod, name.c_str()), "cuModuleGetFunction", err)) return false;
            if (!drv(D.funcSetAttribute(e.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)e.smem),
                     "cuFuncSetAttribute", err))
                return false;
            if (!drv(D.occupancy(&e.per_sm, e.fn, e.TB, e.smem),
                     "cuOccupancyMaxActiveBlocksPerMultiprocessor", err))
                return false;
            g_entries.push_back(e);
            ids.push_back((int)g_entries.size() - 1);
        }
        for (size_t q = 0; q < pairs.size(); q++) {
            const DevPass& p = passes[pairs[q]];
            JitEntry e;
            e.device = dev;
            e.TB = 1 << p.tb_bits;
            e.E = 1 << (p.Tp - p.tb_bits);
            e.smem = (size_t)2 * e.TB * e.E * sizeof(float2);
            const std::string name = "esc_jit_pair" + std::to_string(q);
            if (!drv(D.moduleGetFunction(&e.fn, mod, name.c_str()), "cuModuleGetFunction", err)) return false;
            if (!drv(D.funcSetAttribute(e.fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)e.smem),
                     "cuFuncSetAttribute", err))
                return false;
            if (!drv(D.occupancy(&e.per_sm, e.fn, e.TB, e.smem), "cuOccupancyMaxActiveBlocksPerMultiprocessor", err))
                return false;
            g_entries.push_back(e);
            ids.push_back((int)g_entries.size() - 1);
        }
        it = g_cache.emplace(key, ids).first;
    }
    for (size_t k = 0; k < which.size(); k++) passes[which[k]].jit = it->second[k];
    for (size_t q = 0; q < pairs.size(); q++) passes[pairs[q]].jit_pair = it->second[which.size() + q];
    return true;
}

int jit_launch(const DevPass& p, const escdev::PassTab& pt, const void* diag, const void* in, void* out, int64_t D,
               int sms, cudaStream_t s, const int* active) {
    JitEntry e;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (p.jit < 0 || p.jit >= (int)g_entries.size()) throw std::invalid_argument("no specialised kernel for this pass");
        e = g_entries[p.jit];
    }
    const long long ntiles = (long long)(D >> p.Tp);
    const long long g = std::min<long long>(ntiles, (long long)sms * std::max(e.per_sm, 1));
    if (g <= 0) return 0;
    escdev::PassTab tab = pt;
    const float* dg = (const float*)diag;
    const float2* vin = (const float2*)in;
    float2* vout = (float2*)out;
    long long nt = ntiles;
    const int* act = active;
    void* args[] = {&tab, &dg, &vin, &vout, &nt, &act};
    std::string err;
    if (!drv(driver().launchKernel(e.fn, (unsigned)g, 1, 1, (unsigned)e.TB, 1, 1, (unsigned)e.smem, (CUstream)s, args, nullptr),
             "cuLaunchKernel", err))
        throw CudaError(err);
    return (int)g;
}

int jit_pair_launch(const DevPass& a, const escdev::PassTab& pa, const escdev::PassTab& pb, const escdev::PairTab& st,
                    const void* diag, const void* in, void* out, int64_t D, int sms, cudaStream_t s, const int* active) {
    (void)D;
    JitEntry e;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (a.jit_pair < 0 || a.jit_pair >= (int)g_entries.size()) throw std::invalid_argument("no specialised pair kernel");
        e = g_entries[a.jit_pair];
    }
    const long long items = (2 * st.nslab) << st.inner;
    const long long g = std::min<long long>(items, (long long)sms * std::max(e.per_sm, 1));
    if (g <= 0) return 0;
    escdev::PassTab ta = pa, tb = pb;
    escdev::PairTab tp = st;
    const float* dg = (const float*)diag;
    const float2* vin = (const float2*)in;
    float2* vout = (float2*)out;
    const int* act = active;
    void* args[] = {&ta, &tb, &tp, &dg, &vin, &vout, &act};
    std::string err;
    if (!drv(driver().launchCooperative(e.fn, (unsigned)g, 1, 1, (unsigned)e.TB, 1, 1, (unsigned)e.smem, (CUstream)s, args),
             "cuLaunchCooperativeKernel", err))
        throw CudaError(err);
    return (int)g;
}

}  // namespace esc
