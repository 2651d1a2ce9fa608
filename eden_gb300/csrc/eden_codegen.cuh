// Run-time code generation for the windowed kernels.
//
// The reference writes C for each cell type of the model and compiles it
// with gcc at set-up (eden/Eden.cpp:7017-7180).  Here edenGpuCreate writes
// CUDA for the model's mechanisms -- one straight-line channel-current
// routine per distinct channel set of the non-flat compartments -- prepends
// it to the library's own kernel sources (embedded at build time from
// eden_math.cuh, eden_kernels.cuh and eden_window.cuh) and compiles the lot
// for sm_103a with NVRTC.  The generated routines perform the same float
// operations in the same order as the table-driven loop they replace, so the
// results are identical; the compiled kernels are loaded with
// cudaLibraryLoadData and launched like the built-in ones.  NVRTC is loaded
// with dlopen, so the library still loads (and falls back to its built-in
// kernels) where it is absent.  Compiled libraries are cached per device and
// source for the life of the process.
#pragma once
#include <dlfcn.h>
#include <nvrtc.h>

#include <chrono>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "_rtc_src.inc"

namespace eden_codegen {

struct Nvrtc {
    bool ok = false;
    std::string why;
    nvrtcResult (*create)(nvrtcProgram *, const char *, const char *, int, const char *const *, const char *const *);
    nvrtcResult (*add_name)(nvrtcProgram, const char *);
    nvrtcResult (*compile)(nvrtcProgram, int, const char *const *);
    nvrtcResult (*log_size)(nvrtcProgram, size_t *);
    nvrtcResult (*log)(nvrtcProgram, char *);
    nvrtcResult (*lowered)(nvrtcProgram, const char *, const char **);
    nvrtcResult (*cubin_size)(nvrtcProgram, size_t *);
    nvrtcResult (*cubin)(nvrtcProgram, char *);
    nvrtcResult (*destroy)(nvrtcProgram *);
    const char *(*err)(nvrtcResult);
};

inline Nvrtc &nvrtc() {
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        void *h = nullptr;
        for (const char *name : {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"})
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) {
            n.why = "libnvrtc.so.13 not found";
            return;
        }
        bool all = true;
        auto sym = [&](auto &fp, const char *s) {
            fp = reinterpret_cast<std::remove_reference_t<decltype(fp)>>(dlsym(h, s));
            all = all && fp;
        };
        sym(n.create, "nvrtcCreateProgram");
        sym(n.add_name, "nvrtcAddNameExpression");
        sym(n.compile, "nvrtcCompileProgram");
        sym(n.log_size, "nvrtcGetProgramLogSize");
        sym(n.log, "nvrtcGetProgramLog");
        sym(n.lowered, "nvrtcGetLoweredName");
        sym(n.cubin_size, "nvrtcGetCUBINSize");
        sym(n.cubin, "nvrtcGetCUBIN");
        sym(n.destroy, "nvrtcDestroyProgram");
        sym(n.err, "nvrtcGetErrorString");
        n.ok = all;
        if (!all) n.why = "libnvrtc lacks an entry point";
    });
    return n;
}

// Kernels compiled for one model.
struct Kernels {
    const void *inputs = nullptr, *cells = nullptr, *deliver = nullptr;
};

// One straight-line routine per channel set: for set `sig` it adds the
// channel currents of a non-flat compartment to Ich and Gch exactly as the
// table-driven loop of forest_window does (fopen = product of gate values
// to their instances, then (g*(E - v)*1e-5)*A and (g*1e-5)*A).
inline std::string channel_routines(const EdenGpuChannelType *types, const std::vector<std::vector<int>> &sets) {
    std::string s;
    char b[256];
    s += "namespace eden {\n#define EDEN_RTC_CHANNELS 1\n";
    s += "__device__ __forceinline__ bool rtc_channels(int sig, const float *q, const float *CHG, const float *CHE,\n"
         "                                             int c0, float v, float A, float &Ich, float &Gch) {\n"
         "    switch (sig) {\n";
    for (size_t k = 0; k < sets.size(); k++) {
        snprintf(b, sizeof(b), "    case %d: {\n", (int)k);
        s += b;
        int qoff = 0;
        for (size_t c = 0; c < sets[k].size(); c++) {
            const EdenGpuChannelType &t = types[sets[k][c]];
            s += "        {\n            float fopen = 1.0f;\n";
            for (int g = 0; g < t.n_gates; g++) {
                for (int r = 0; r < t.gate_instances[g]; r++) {
                    snprintf(b, sizeof(b), "            fopen = fopen * q[%d];\n", qoff + g);
                    s += b;
                }
            }
            qoff += t.n_gates;
            snprintf(b, sizeof(b),
                     "            const float gs = CHG[c0 + %d] * fopen;\n"
                     "            Ich += (gs * (CHE[c0 + %d] - v) * 1e-5f) * A;\n"
                     "            Gch += (gs * 1e-5f) * A;\n        }\n",
                     (int)c, (int)c);
            s += b;
        }
        s += "        return true;\n    }\n";
    }
    s += "    default: return false;\n    }\n}\n}  // namespace eden\n";
    return s;
}

// The kinds of inputs and targets the model has: the generated build
// compiles only their code (the EDEN_KIND_* switches of eden_kernels.cuh).
struct Kinds {
    bool pulse = false, sine = false, ramp = false, pois = false, timed = false, syn = false, expone = false,
         exptwo = false, forest = false, izh = false, gateforms = false, clamp = false, gap = false, alpha = false,
         current = false;
};

inline std::string kind_defines(const Kinds &k) {
    std::string s;
    auto def = [&](const char *name, bool on) { s += std::string("#define ") + name + (on ? " 1\n" : " 0\n"); };
    def("EDEN_KIND_PULSE", k.pulse);
    def("EDEN_KIND_GATEFORMS", k.gateforms);
    def("EDEN_KIND_CLAMP", k.clamp);
    def("EDEN_KIND_SINE", k.sine);
    def("EDEN_KIND_RAMP", k.ramp);
    def("EDEN_KIND_POIS", k.pois);
    def("EDEN_KIND_TIMED", k.timed);
    def("EDEN_KIND_SYN", k.syn);
    def("EDEN_KIND_EXPONE", k.expone);
    def("EDEN_KIND_EXPTWO", k.exptwo);
    def("EDEN_KIND_FOREST", k.forest);
    def("EDEN_KIND_IZH", k.izh);
    def("EDEN_KIND_GAP", k.gap);
    def("EDEN_KIND_ALPHA", k.alpha);
    def("EDEN_KIND_CURRENT", k.current);
    return s;
}

// The full source: integer types NVRTC has no headers for, the generated
// routines (plain arithmetic, needing nothing else), then the library's
// kernel sources, which call them where EDEN_RTC_CHANNELS is defined.
inline std::string program_source(const std::string &generated) {
    std::string s =
        "// generated by libeden_gpu for one model\n"
        "typedef signed char int8_t;\ntypedef unsigned char uint8_t;\ntypedef short int16_t;\n"
        "typedef unsigned short uint16_t;\ntypedef int int32_t;\ntypedef unsigned int uint32_t;\n"
        "typedef long long int64_t;\ntypedef unsigned long long uint64_t;\n"
        "typedef decltype(sizeof(0)) size_t;\n" + generated;
    for (const char *part : kRtcSourceParts) s += part;
    return s;
}

// Compiles `src` for the current device (cached); fills `k`.
inline bool compile(const std::string &src, int device, Kernels &k, std::string &err, double &ms) {
    static std::mutex mu;
    static std::map<std::pair<int, std::string>, Kernels> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto hit = cache.find({device, src});
    if (hit != cache.end()) {
        k = hit->second;
        ms = 0.0;
        return true;
    }
    Nvrtc &n = nvrtc();
    if (!n.ok) {
        err = n.why;
        return false;
    }
    const auto t0 = std::chrono::steady_clock::now();
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        err = "cudaGetDeviceProperties failed";
        return false;
    }
    char arch[64];
    snprintf(arch, sizeof(arch), "--gpu-architecture=sm_%d%da", prop.major, prop.minor);
    nvrtcProgram prog;
    nvrtcResult r = n.create(&prog, src.c_str(), "eden_rtc.cu", 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) {
        err = std::string("nvrtcCreateProgram: ") + n.err(r);
        return false;
    }
    const char *names[3] = {"eden::k_inputs_t", "eden::k_cells_t", "eden::k_deliver_t"};
    for (const char *nm : names) n.add_name(prog, nm);
    const char *opts[] = {arch, "-std=c++17", "-DEDEN_RTC=1", "-lineinfo"};
    r = n.compile(prog, 4, opts);
    if (r != NVRTC_SUCCESS) {
        size_t len = 0;
        n.log_size(prog, &len);
        std::string log(len, '\0');
        if (len) n.log(prog, &log[0]);
        err = std::string("nvrtcCompileProgram: ") + n.err(r) + "\n" + log.substr(0, 4000);
        n.destroy(&prog);
        return false;
    }
    size_t size = 0;
    n.cubin_size(prog, &size);
    std::vector<char> cubin(size);
    n.cubin(prog, cubin.data());
    cudaLibrary_t lib;
    if (cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess) {
        err = "cudaLibraryLoadData failed";
        n.destroy(&prog);
        return false;
    }
    const void **slots[3] = {&k.inputs, &k.cells, &k.deliver};
    for (int i = 0; i < 3; i++) {
        const char *low = nullptr;
        cudaKernel_t kern;
        if (n.lowered(prog, names[i], &low) != NVRTC_SUCCESS || cudaLibraryGetKernel(&kern, lib, low) != cudaSuccess) {
            err = std::string("kernel not found: ") + names[i];
            n.destroy(&prog);
            return false;
        }
        *slots[i] = (const void *)kern;
    }
    n.destroy(&prog);
    cache[{device, src}] = k;
    ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return true;
}

}  // namespace eden_codegen
