// libeden_gpu: C ABI (include/eden_gpu.h) over the simulation kernels.
//
// edenGpuCreate validates the lowered model, builds the device layout
// (breadth-first compartments, inputs sorted by target, source fan-out CSR,
// cell groups for the windowed kernel) and uploads it.  edenGpuRun advances
// the network: per step (EDEN_MODE_PLAIN: four launches a step, as the
// reference runs one OpenMP pass a step) or in windows of K steps
// (EDEN_MODE_BATCHED: one k_window + one k_deliver per window, replayed from
// a captured CUDA graph).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/eden_gpu.h"
#include "eden_kernels.cuh"

using namespace eden;

namespace {

constexpr int kForestNodes = 768;   // largest forest (a larger cell gets a forest of its own)
constexpr int kForestWidth = 64;    // most compartments of a forest at one depth (two per lane)
constexpr int kGraphWindows = 16;  // windows per captured graph

// Host set-up loops whose iterations are independent run on the host's
// threads (at most 16, at least `grain` iterations each), in contiguous
// blocks of the index range; small ranges run inline.
template <typename F>
void parallel_for(int64_t n, F f, int64_t grain = 16384) {
    const int64_t hw = std::max<int64_t>(1, std::min<int64_t>(16, (int64_t)std::thread::hardware_concurrency()));
    const int64_t nthr = std::min<int64_t>(hw, n / grain);
    if (nthr <= 1) {
        for (int64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::vector<std::thread> pool;
    for (int64_t t = 0; t < nthr; t++)
        pool.emplace_back([=, &f] {
            const int64_t a = n * t / nthr, b = n * (t + 1) / nthr;
            for (int64_t i = a; i < b; i++) f(i);
        });
    for (auto &th : pool) th.join();
}

struct Window {
    int64_t step0;
    int32_t K;
};

}  // namespace

struct EdenGpuCtx {
    std::string err;
    int device = 0;
    int mode = EDEN_MODE_PLAIN;
    int K = 1;                 // window length (batched)
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    DevModel d{};
    std::vector<void *> allocs;
    // host copies needed for reads
    int n_target = 0, n_comp_user = 0, n_izh = 0;
    std::vector<int32_t> user_to_internal;   // user target -> internal target
    std::vector<int64_t> syn_internal_of_user;  // user synapse -> internal synapse
    std::vector<uint8_t> h_sy_type;             // internal synapse -> synapse type
    std::vector<SynTypeDev> h_syn_types;
    int64_t n_syn = 0;
    // run state
    int64_t next_step = -3;
    double time = 0.0;          // time of next_step (accumulated in double as the reference does)
    int par = 0, wpar = 0, Kprev = 1;
    double t_prev0 = 0.0;
    int64_t trace_first_unfetched = 1;   // first non-init step not yet fetched
    int64_t trace_cap = 0;
    int32_t n_trace = 0;
    // window table (device + pinned host)
    WindowArgs *d_wtab = nullptr;
    WindowArgs *h_wtab = nullptr;
    WindowTimes *d_wtimes = nullptr;
    WindowTimes *h_wtimes = nullptr;
    float prev_tk[32] = {0};    // step times of the last window run
    int64_t wtab_cap = 0;
    int *d_base = nullptr;      // chunk base read by graph-launched kernels
    int *d_zero = nullptr;      // always 0, for direct launches
    cudaGraphExec_t graph = nullptr;
    int grid_inputs = 0, grid_targets = 0, grid_hines = 0, grid_deliver = 0, grid_window = 0;
    int n_sm_unused = 0;
    int smem_per_sm = 0, smem_optin = 0;   // bytes
    int gcap = 0, forest_cap = 0;           // largest cell / compartments per staged forest
    bool smem_window = false;              // groups fit shared memory
    int max_cell_blocks = 0;               // most blocks of a k_cells_t launch
    std::vector<int64_t> h_ext_step;       // logging steps of the spike sources' events
    size_t smem_hines = 0;
    struct CellClass { int cta_begin, cta_end; size_t smem; };
    std::vector<CellClass> classes;        // k_cells_t launches of one window
    double last_ms = 0.0;
    int64_t last_launches = 0;
    // kernel timing: an event pair per launch of the current run
    bool kernel_timing = false;
    std::vector<cudaEvent_t> tev;
    std::vector<int> tev_kind;
    size_t tev_used = 0;
    double k_ms[EDEN_KERNEL_KINDS] = {0};
    int64_t k_n[EDEN_KERNEL_KINDS] = {0};
    int sticky_status = 0;
    // set when a run failed after its kernels began to change the device
    // state: the host clock and the device state may then disagree, so
    // later runs are refused
    bool broken = false;
    int64_t n_f64_cells = 0;    // cells whose cable solve runs in double precision
    bool launched = false;      // the current run has issued a kernel
    // edenGpuRunStaticScratch: device addresses of the static arrays, looked
    // up on the context's first such call (the context's device current)
    float *static_gp = nullptr;
    WindowArgs *static_tab = nullptr;
    WindowTimes *static_times = nullptr;
    // the windowed kernels launched: the built-in ones or those compiled for
    // this model at creation (eden_codegen.cuh)
    const void *fn_inputs = nullptr, *fn_cells = nullptr, *fn_deliver = nullptr;
    bool codegen_used = false;
    std::string codegen_source, codegen_note;
    double codegen_ms = 0.0;

    int fail(int code, const char *fmt, ...) {
        char buf[1024];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
};

#define CUDA_TRY(ctx, call)                                                                         \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return (ctx)->fail(e_ == cudaErrorMemoryAllocation ? EDEN_GPU_E_NOMEM : EDEN_GPU_E_CUDA, \
                               "%s failed: %s", #call, cudaGetErrorString(e_));                     \
    } while (0)

#include "eden_window.cuh"
#include "eden_codegen.cuh"

namespace {
// Launch of a kernel given by handle (a built-in __global__ function or a
// kernel loaded from the model's compiled library).
template <typename... A>
cudaError_t launch_k(const void *fn, int grid, int block, size_t smem, cudaStream_t s, A... args) {
    void *argv[] = {(void *)&args...};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), argv, smem, s);
}
}  // namespace

// ---------------------------------------------------------------------------
namespace {

template <typename T>
int upload(EdenGpuCtx *ctx, T **dst, const T *src, size_t n) {
    size_t bytes = sizeof(T) * (n > 0 ? n : 1);
    void *p = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&p, bytes));
    ctx->allocs.push_back(p);
    if (src && n) {
        CUDA_TRY(ctx, cudaMemcpy(p, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    } else {
        CUDA_TRY(ctx, cudaMemset(p, 0, bytes));
    }
    *dst = (T *)p;
    return 0;
}

template <typename T>
int upload_vec(EdenGpuCtx *ctx, T **dst, const std::vector<T> &v) {
    return upload(ctx, dst, v.data(), v.size());
}

template <typename T>
int upload_c(EdenGpuCtx *ctx, const T **dst, const std::vector<T> &v) {
    T *p = nullptr;
    int rc = upload(ctx, &p, v.data(), v.size());
    *dst = p;
    return rc;
}

#define TRY(x)                  \
    do {                        \
        int rc_ = (x);          \
        if (rc_) return rc_;    \
    } while (0)

bool finite_pos(float x) { return std::isfinite(x) && x > 0.0f; }

// synapse kinds whose state is a current (blocks flagged BK_CURRENT)
bool current_kind(int kind) { return kind == EDEN_SYN_ALPHA_CURRENT || kind == EDEN_SYN_EXPONE_CURRENT; }


int validate(EdenGpuCtx *ctx, const EdenGpuModel *m) {
    if (m->abi_version != EDEN_GPU_ABI_VERSION)
        return ctx->fail(EDEN_GPU_E_INVALID, "ABI version %d, library is %d", m->abi_version, EDEN_GPU_ABI_VERSION);
    if (!(m->dt > 0.0f) || !std::isfinite(m->dt)) return ctx->fail(EDEN_GPU_E_INVALID, "dt must be positive");
    if (m->n_phys < 0 || m->n_comp < 0 || m->n_izh < 0 || m->n_syn < 0 || m->n_pois < 0 || m->n_pulse < 0)
        return ctx->fail(EDEN_GPU_E_INVALID, "negative count");
    if ((int64_t)m->n_comp + m->n_izh > INT32_MAX / 2) return ctx->fail(EDEN_GPU_E_INVALID, "too many targets");
    if (m->n_syn > INT32_MAX / 2 || m->n_pois > INT32_MAX / 2)
        return ctx->fail(EDEN_GPU_E_INVALID, "too many synapses");
    if (m->n_chan_types > kMaxChanTypes || m->n_syn_types > kMaxSynTypes)
        return ctx->fail(EDEN_GPU_E_INVALID, "too many channel or synapse types");
    if (m->cable_solver != EDEN_CABLE_BWD_EULER && m->cable_solver != EDEN_CABLE_FWD_EULER)
        return ctx->fail(EDEN_GPU_E_INVALID, "unknown cable solver %d", m->cable_solver);
    if (m->phys_comp_off[0] != 0 || m->phys_comp_off[m->n_phys] != m->n_comp)
        return ctx->fail(EDEN_GPU_E_INVALID, "phys_comp_off must span [0, n_comp]");
    for (int c = 0; c < m->n_phys; c++) {
        int a = m->phys_comp_off[c], b = m->phys_comp_off[c + 1];
        if (b <= a) return ctx->fail(EDEN_GPU_E_INVALID, "cell %d has no compartments", c);
        if (m->comp_parent[a] != -1) return ctx->fail(EDEN_GPU_E_INVALID, "cell %d: compartment 0 must be the root", c);
        for (int i = a + 1; i < b; i++) {
            int p = m->comp_parent[i];
            if (p < 0 || p >= i - a)
                return ctx->fail(EDEN_GPU_E_INVALID, "cell %d compartment %d: parent %d must precede it", c, i - a, p);
            if (!finite_pos(m->comp_r_axial[i])) return ctx->fail(EDEN_GPU_E_INVALID, "compartment %d: bad axial resistance", i);
        }
    }
    for (int i = 0; i < m->n_comp; i++) {
        if (!finite_pos(m->comp_c[i])) return ctx->fail(EDEN_GPU_E_INVALID, "compartment %d: bad capacitance", i);
        if (!std::isfinite(m->comp_area[i]) || !std::isfinite(m->comp_inv_rc[i]) || !std::isfinite(m->comp_v0[i]))
            return ctx->fail(EDEN_GPU_E_INVALID, "compartment %d: non-finite constant", i);
    }
    if (m->comp_chan_off[0] != 0) return ctx->fail(EDEN_GPU_E_INVALID, "comp_chan_off[0] != 0");
    for (int i = 0; i < m->n_comp; i++)
        if (m->comp_chan_off[i + 1] < m->comp_chan_off[i]) return ctx->fail(EDEN_GPU_E_INVALID, "comp_chan_off not monotone");
    int n_chan = m->comp_chan_off[m->n_comp];
    for (int ch = 0; ch < n_chan; ch++)
        if (m->chan_type[ch] < 0 || m->chan_type[ch] >= m->n_chan_types)
            return ctx->fail(EDEN_GPU_E_INVALID, "channel %d: bad type", ch);
    for (int k = 0; k < m->n_chan_types; k++) {
        const EdenGpuChannelType &t = m->chan_types[k];
        if (t.n_gates < 0 || t.n_gates > EDEN_MAX_GATES) return ctx->fail(EDEN_GPU_E_INVALID, "channel type %d: gate count", k);
        for (int g = 0; g < t.n_gates; g++) {
            if (t.gate_instances[g] < 0 || t.gate_instances[g] > 16) return ctx->fail(EDEN_GPU_E_INVALID, "gate instances");
            if (t.gate_kind[g] < 0 || t.gate_kind[g] >= EDEN_GATE_KINDS)
                return ctx->fail(EDEN_GPU_E_INVALID, "channel type %d gate %d: gate kind %d", k, g, t.gate_kind[g]);
            const int gk = t.gate_kind[g];
            if (gk != EDEN_GATE_TAUINF && gk != EDEN_GATE_INSTANTANEOUS &&
                (t.fwd_kind[g] < 0 || t.fwd_kind[g] > 2 || t.rev_kind[g] < 0 || t.rev_kind[g] > 2))
                return ctx->fail(EDEN_GPU_E_INVALID, "channel type %d gate %d: rate kind", k, g);
            if ((gk == EDEN_GATE_TAUINF || gk == EDEN_GATE_RATESTAU || gk == EDEN_GATE_RATESTAUINF) &&
                (t.tau_kind[g] < 0 || t.tau_kind[g] > EDEN_RATE_FIXED))
                return ctx->fail(EDEN_GPU_E_INVALID, "channel type %d gate %d: timeCourse form", k, g);
            if ((gk == EDEN_GATE_TAUINF || gk == EDEN_GATE_RATESINF || gk == EDEN_GATE_RATESTAUINF ||
                 gk == EDEN_GATE_INSTANTANEOUS) &&
                (t.inf_kind[g] < 0 || t.inf_kind[g] > EDEN_RATE_FIXED))
                return ctx->fail(EDEN_GPU_E_INVALID, "channel type %d gate %d: steadyState form", k, g);
        }
    }
    int64_t nt = (int64_t)m->n_comp + m->n_izh;
    if (nt == 0) return ctx->fail(EDEN_GPU_E_INVALID, "empty network");
    if (m->n_izh > 0 && !m->izh_params) return ctx->fail(EDEN_GPU_E_INVALID, "point-neuron parameters missing");
    for (int k = 0; k < m->n_izh; k++) {
        const int kind = m->izh_kind ? m->izh_kind[k] : EDEN_POINT_IZH2007;
        if (kind < 0 || kind >= EDEN_POINT_KINDS)
            return ctx->fail(EDEN_GPU_E_INVALID, "point neuron %d: kind %d unknown", k, kind);
        for (int f = 0; f < EDEN_POINT_PARAMS; f++)
            if (!std::isfinite(m->izh_params[EDEN_POINT_PARAMS * (int64_t)k + f]))
                return ctx->fail(EDEN_GPU_E_INVALID, "point neuron %d: parameter %d not finite", k, f);
    }
    if (m->n_src < m->n_phys + m->n_izh)
        return ctx->fail(EDEN_GPU_E_INVALID, "need one spike source per cell (n_src %d, cells %d)", m->n_src,
                         m->n_phys + m->n_izh);
    {
        int with_target = 0;
        for (int s = 0; s < m->n_src; s++) {
            if (m->src_target[s] == -1) continue;  // a spike list or generator
            if (m->src_target[s] < 0 || m->src_target[s] >= nt) return ctx->fail(EDEN_GPU_E_INVALID, "source %d: bad target", s);
            with_target++;
        }
        if (with_target != m->n_phys + m->n_izh)
            return ctx->fail(EDEN_GPU_E_INVALID, "need one spike source per cell (%d with a target, cells %d)",
                             with_target, m->n_phys + m->n_izh);
    }
    if (m->n_ext < 0 || m->n_ext > INT32_MAX / 2 || (m->n_ext > 0 && (!m->ext_src || !m->ext_step)))
        return ctx->fail(EDEN_GPU_E_INVALID, "bad spike-source event list");
    for (int64_t k = 0; k < m->n_ext; k++) {
        const int s = m->ext_src[k];
        if (s < 0 || s >= m->n_src || m->src_target[s] != -1)
            return ctx->fail(EDEN_GPU_E_INVALID, "spike-source event %lld: source %d is not a source without target",
                             (long long)k, s);
        if (m->ext_step[k] < 2 || m->ext_step[k] > INT32_MAX || (k > 0 && m->ext_step[k] < m->ext_step[k - 1]))
            return ctx->fail(EDEN_GPU_E_INVALID, "spike-source event %lld: steps must be >= 2 and sorted", (long long)k);
    }
    for (int k = 0; k < m->n_syn_types; k++) {
        const EdenGpuSynapseType &t = m->syn_types[k];
        if (t.kind < EDEN_SYN_EXPONE || t.kind > EDEN_SYN_BLOCKING_PLASTIC)
            return ctx->fail(EDEN_GPU_E_INVALID, "synapse type kind");
        if (t.kind == EDEN_SYN_BLOCKING_PLASTIC &&
            (!std::isfinite(t.release_prob) || !(t.tau_rec >= 0.0f) || !(t.tau_fac >= 0.0f) ||
             !std::isfinite(t.block_ratio) || !std::isfinite(t.block_volt) || !std::isfinite(t.tau_rec) ||
             !std::isfinite(t.tau_fac)))
            return ctx->fail(EDEN_GPU_E_INVALID, "synapse type %d: plasticity or block parameters", k);
        const bool two = t.kind == EDEN_SYN_EXPTWO || t.kind == EDEN_SYN_BLOCKING_PLASTIC;
        if (!finite_pos(t.tau_decay) || (two && !finite_pos(t.tau_rise)))
            return ctx->fail(EDEN_GPU_E_INVALID, "synapse type %d: time constants", k);
    }
    for (int64_t s = 0; s < m->n_syn; s++) {
        if (m->syn_target[s] < 0 || m->syn_target[s] >= nt || m->syn_type[s] < 0 || m->syn_type[s] >= m->n_syn_types ||
            m->syn_src[s] < 0 || m->syn_src[s] >= m->n_src)
            return ctx->fail(EDEN_GPU_E_INVALID, "synapse %lld: index out of range", (long long)s);
        if (!(m->syn_delay[s] >= 0.0f) || !std::isfinite(m->syn_delay[s]))
            return ctx->fail(EDEN_GPU_E_INVALID, "synapse %lld: bad delay", (long long)s);
    }
    for (int64_t k = 0; k < m->n_pois; k++)
        if (m->pois_target[k] < 0 || m->pois_target[k] >= nt || m->pois_type[k] < 0 || m->pois_type[k] >= m->n_syn_types ||
            m->pois_src[k] < 0 || m->pois_src[k] >= m->n_src || !finite_pos(m->pois_rate[k]))
            return ctx->fail(EDEN_GPU_E_INVALID, "poisson input %lld: bad field", (long long)k);
    if (m->n_timed < 0 || m->n_timed > INT32_MAX / 2 ||
        (m->n_timed > 0 && (!m->timed_target || !m->timed_type || !m->timed_weight || !m->timed_off || !m->timed_step)))
        return ctx->fail(EDEN_GPU_E_INVALID, "bad timed-input arrays");
    if (m->n_timed > 0 && m->timed_off[0] != 0) return ctx->fail(EDEN_GPU_E_INVALID, "timed_off[0] != 0");
    for (int64_t k = 0; k < m->n_timed; k++) {
        if (m->timed_target[k] < 0 || m->timed_target[k] >= nt || m->timed_type[k] < 0 ||
            m->timed_type[k] >= m->n_syn_types || m->timed_off[k + 1] < m->timed_off[k] || !std::isfinite(m->timed_weight[k]))
            return ctx->fail(EDEN_GPU_E_INVALID, "timed input %lld: bad field", (long long)k);
        for (int64_t j = m->timed_off[k]; j < m->timed_off[k + 1]; j++)
            if (m->timed_step[j] < 1 || (j > m->timed_off[k] && m->timed_step[j] <= m->timed_step[j - 1]))
                return ctx->fail(EDEN_GPU_E_INVALID, "timed input %lld: steps must be >= 1 and increasing", (long long)k);
    }
    for (int64_t k = 0; k < m->n_pulse; k++)
        if (m->pulse_target[k] < 0 || m->pulse_target[k] >= nt)
            return ctx->fail(EDEN_GPU_E_INVALID, "pulse %lld: bad target", (long long)k);
    if (m->n_wave < 0) return ctx->fail(EDEN_GPU_E_INVALID, "n_wave must be >= 0");
    if (m->n_wave > 0 && (!m->wave_target || !m->wave_shape || !m->wave_params || !m->wave_weight))
        return ctx->fail(EDEN_GPU_E_INVALID, "waveform inputs: null array");
    for (int64_t k = 0; k < m->n_wave; k++) {
        if (m->wave_target[k] < 0 || m->wave_target[k] >= nt)
            return ctx->fail(EDEN_GPU_E_INVALID, "waveform input %lld: bad target", (long long)k);
        if (m->wave_shape[k] < 0 || m->wave_shape[k] >= EDEN_WAVE_SHAPES)
            return ctx->fail(EDEN_GPU_E_INVALID, "waveform input %lld: unknown shape %d", (long long)k,
                             m->wave_shape[k]);
        bool finite = std::isfinite(m->wave_weight[k]);
        for (int j = 0; j < EDEN_WAVE_PARAMS; j++) finite = finite && std::isfinite(m->wave_params[EDEN_WAVE_PARAMS * k + j]);
        if (!finite) return ctx->fail(EDEN_GPU_E_INVALID, "waveform input %lld: non-finite parameter", (long long)k);
    }
    if (m->n_clamp < 0) return ctx->fail(EDEN_GPU_E_INVALID, "n_clamp must be >= 0");
    if (m->n_clamp > 0 && (!m->clamp_target || !m->clamp_params || !m->clamp_weight))
        return ctx->fail(EDEN_GPU_E_INVALID, "voltage clamps: null array");
    for (int64_t k = 0; k < m->n_clamp; k++) {
        const float *p = m->clamp_params + EDEN_CLAMP_PARAMS * k;
        if (m->clamp_target[k] < 0 || m->clamp_target[k] >= nt)
            return ctx->fail(EDEN_GPU_E_INVALID, "voltage clamp %lld: bad target", (long long)k);
        if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[5]) || p[5] == 0.0f ||
            !std::isfinite(m->clamp_weight[k]) || std::isinf(p[2]) || std::isinf(p[3]) || std::isinf(p[4]))
            return ctx->fail(EDEN_GPU_E_INVALID, "voltage clamp %lld: bad parameter", (long long)k);
    }
    if (m->pois_rng_base)
        for (int64_t k = 0; k < m->n_pois; k++)
            if (m->pois_rng_base[k] < 0)
                return ctx->fail(EDEN_GPU_E_INVALID, "Poisson input %lld: negative random-call id", (long long)k);
    if (m->n_gap < 0) return ctx->fail(EDEN_GPU_E_INVALID, "n_gap must be >= 0");
    if (m->n_gap > 0 && (!m->gap_target || !m->gap_peer || !m->gap_conductance || !m->gap_weight))
        return ctx->fail(EDEN_GPU_E_INVALID, "gap junctions: null array");
    for (int64_t k = 0; k < m->n_gap; k++) {
        if (m->gap_target[k] < 0 || m->gap_target[k] >= m->n_comp || m->gap_peer[k] < 0 || m->gap_peer[k] >= m->n_comp)
            return ctx->fail(EDEN_GPU_E_INVALID, "gap junction %lld: ends must be compartments of physical cells",
                             (long long)k);
        if (!std::isfinite(m->gap_conductance[k]) || !std::isfinite(m->gap_weight[k]))
            return ctx->fail(EDEN_GPU_E_INVALID, "gap junction %lld: non-finite conductance or weight", (long long)k);
    }
    for (int64_t k = 0; k < m->n_pois; k++)
        if (m->syn_types[m->pois_type[k]].kind == EDEN_SYN_BLOCKING_PLASTIC)
            return ctx->fail(EDEN_GPU_E_INVALID, "Poisson input %lld: blocking-plastic synapses on connections only",
                             (long long)k);
    for (int64_t k = 0; k < m->n_timed; k++)
        if (m->syn_types[m->timed_type[k]].kind == EDEN_SYN_BLOCKING_PLASTIC)
            return ctx->fail(EDEN_GPU_E_INVALID, "timed input %lld: blocking-plastic synapses on connections only",
                             (long long)k);
    if (m->n_graded < 0) return ctx->fail(EDEN_GPU_E_INVALID, "n_graded must be >= 0");
    if (m->n_graded > 0 && (!m->graded_target || !m->graded_peer || !m->graded_params || !m->graded_weight))
        return ctx->fail(EDEN_GPU_E_INVALID, "graded synapses: null array");
    for (int64_t k = 0; k < m->n_graded; k++) {
        if (m->graded_target[k] < 0 || m->graded_target[k] >= m->n_comp || m->graded_peer[k] < 0 ||
            m->graded_peer[k] >= m->n_comp)
            return ctx->fail(EDEN_GPU_E_INVALID, "graded synapse %lld: ends must be compartments of physical cells",
                             (long long)k);
        const float *p = m->graded_params + (size_t)EDEN_GRADED_PARAMS * k;
        for (int j = 0; j < EDEN_GRADED_PARAMS; j++)
            if (!std::isfinite(p[j])) return ctx->fail(EDEN_GPU_E_INVALID, "graded synapse %lld: non-finite parameter", (long long)k);
        if (p[1] == 0.0f || !(p[2] > 0.0f) || !std::isfinite(m->graded_weight[k]))
            return ctx->fail(EDEN_GPU_E_INVALID, "graded synapse %lld: delta must be non-zero, k positive", (long long)k);
    }
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" int edenGpuAbiVersion(void) { return EDEN_GPU_ABI_VERSION; }

extern "C" const char *edenGpuLastError(EdenGpuCtx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" int64_t edenGpuGeneratedSource(EdenGpuCtx *ctx, char *buf, int64_t cap) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    if (!ctx->codegen_used) return 0;
    const std::string &src = ctx->codegen_source;
    if (buf && cap > 0) {
        const size_t k = std::min<size_t>(src.size(), (size_t)(cap - 1));
        memcpy(buf, src.data(), k);
        buf[k] = '\0';
    }
    return (int64_t)src.size();
}

extern "C" void edenGpuDestroy(EdenGpuCtx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    for (void *p : ctx->allocs) cudaFree(p);
    for (cudaEvent_t e : ctx->tev) cudaEventDestroy(e);
    if (ctx->h_wtab) cudaFreeHost(ctx->h_wtab);
    if (ctx->h_wtimes) cudaFreeHost(ctx->h_wtimes);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static int build_and_upload(EdenGpuCtx *ctx, const EdenGpuModel *m, const EdenGpuOptions *opt) {
    const int n_comp = m->n_comp, n_izh = m->n_izh, n_phys = m->n_phys;
    const int nt = n_comp + n_izh;
    // set-up phase timing, printed with EDEN_GPU_VERBOSE
    const bool verbose = getenv("EDEN_GPU_VERBOSE") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    std::string timing;
    auto phase = [&](const char *next) {
        const auto now = std::chrono::steady_clock::now();
        char b[64];
        snprintf(b, sizeof(b), " %.1f ms, then %s:", std::chrono::duration<double, std::milli>(now - t_last).count(), next);
        timing += b;
        t_last = now;
    };
    timing = "cells:";
    const int n_cells = m->n_src;
    const float dt = m->dt;
    ctx->n_target = nt;
    ctx->n_comp_user = n_comp;
    ctx->n_izh = n_izh;

    // ---- cells in gid order (one spike source per cell)
    std::vector<int32_t> comp_cell(n_comp);
    for (int c = 0; c < n_phys; c++)
        for (int i = m->phys_comp_off[c]; i < m->phys_comp_off[c + 1]; i++) comp_cell[i] = c;
    std::vector<int32_t> cell_phys(n_cells, -1), cell_izh(n_cells, -1), cell_n(n_cells, 1);
    {
        std::vector<char> seen_phys(n_phys, 0), seen_izh(n_izh, 0);
        for (int g = 0; g < n_cells; g++) {
            int ut = m->src_target[g];
            if (ut < 0) {
                cell_n[g] = 0;  // a spike list or generator: no target
                continue;
            }
            if (ut < n_comp) {
                int c = comp_cell[ut];
                if (seen_phys[c]) return ctx->fail(EDEN_GPU_E_INVALID, "cell %d has two spike sources", c);
                seen_phys[c] = 1;
                cell_phys[g] = c;
                cell_n[g] = m->phys_comp_off[c + 1] - m->phys_comp_off[c];
            } else {
                int k = ut - n_comp;
                if (seen_izh[k]) return ctx->fail(EDEN_GPU_E_INVALID, "izhikevich cell %d has two spike sources", k);
                seen_izh[k] = 1;
                cell_izh[g] = k;
            }
        }
    }
    // per-cell work estimate (inputs dominate) to balance groups
    std::vector<int64_t> n_in_user(nt, 0);
    for (int64_t s = 0; s < m->n_syn; s++) n_in_user[m->syn_target[s]]++;
    for (int64_t k = 0; k < m->n_pois; k++) n_in_user[m->pois_target[k]]++;
    for (int64_t k = 0; k < m->n_timed; k++) n_in_user[m->timed_target[k]]++;
    for (int64_t k = 0; k < m->n_pulse; k++) n_in_user[m->pulse_target[k]]++;
    for (int64_t k = 0; k < m->n_wave; k++) n_in_user[m->wave_target[k]]++;
    for (int64_t k = 0; k < m->n_clamp; k++) n_in_user[m->clamp_target[k]] += 2;
    for (int64_t k = 0; k < m->n_gap; k++) n_in_user[m->gap_target[k]]++;
    for (int64_t k = 0; k < m->n_graded; k++) n_in_user[m->graded_target[k]]++;
    std::vector<double> cost(n_cells, 0.0);
    double total = 0;
    int max_cell = 1;
    for (int g = 0; g < n_cells; g++) {
        double c = 0;
        if (cell_phys[g] >= 0) {
            int a = m->phys_comp_off[cell_phys[g]], b = m->phys_comp_off[cell_phys[g] + 1];
            for (int i = a; i < b; i++)
                c += 6.0 + n_in_user[i] + 8.0 * (m->comp_chan_off[i + 1] - m->comp_chan_off[i]);
            max_cell = std::max(max_cell, b - a);
        } else if (cell_izh[g] >= 0) {
            c = 6.0 + n_in_user[n_comp + cell_izh[g]];
        }
        cost[g] = c;
        total += c;
    }

    // ---- diagonal dominance: row i of a cell's backward-Euler cable matrix
    // (eden/Eden.cpp:6114-6225) has 1 + dt (G_i / C_i + sum_j 1/(R_ij C_i))
    // on the diagonal and dt / (R_ij C_i) off it, so it dominates whenever
    // the membrane conductance G_i >= 0.  G_i is a sum of channel
    // conductances (gbase fopen, fopen >= 0) and synaptic / input
    // conductances (weight times an exposure whose sign is that of gbase
    // times the event jump), so a cell can lose dominance only through a
    // negative channel density, synaptic gbase, expTwo jump or weight.  Such
    // cells are flagged: their elimination runs in double precision.
    // (the forward-Euler update solves nothing: no cell is flagged)
    std::vector<char> cell_f64(n_phys, 0);
    if (m->cable_solver == EDEN_CABLE_BWD_EULER) {
        auto syn_sign = [&](int type, float w) {
            const EdenGpuSynapseType &st = m->syn_types[type];
            if (current_kind(st.kind)) return 1.0f;  // a current: no conductance on the diagonal
            float sg = st.gbase * w;
            if (st.kind == EDEN_SYN_EXPTWO || st.kind == EDEN_SYN_BLOCKING_PLASTIC)
                sg *= st.waveform_factor * st.weight_prop;
            return sg;
        };
        auto flag_comp = [&](int32_t t) { if (t >= 0 && t < n_comp) cell_f64[comp_cell[t]] = 1; };
        for (int i = 0; i < n_comp; i++)
            for (int ch = m->comp_chan_off[i]; ch < m->comp_chan_off[i + 1]; ch++)
                if (m->chan_gbase[ch] < 0.0f) flag_comp(i);
        for (int64_t k = 0; k < m->n_syn; k++)
            if (syn_sign(m->syn_type[k], m->syn_weight[k]) < 0.0f) flag_comp(m->syn_target[k]);
        for (int64_t k = 0; k < m->n_pois; k++)
            if (syn_sign(m->pois_type[k], m->pois_weight[k]) < 0.0f) flag_comp(m->pois_target[k]);
        for (int64_t k = 0; k < m->n_timed; k++)
            if (syn_sign(m->timed_type[k], m->timed_weight[k]) < 0.0f) flag_comp(m->timed_target[k]);
    }
    ctx->n_f64_cells = 0;
    for (int c = 0; c < n_phys; c++) ctx->n_f64_cells += cell_f64[c];

    phase("order");
    // ---- schedule order: physical cells by tree depth (then size), then point
    // neurons, so that a CTA's warps finish their cable solves together; the
    // cells flagged for a double-precision solve after the others, in forests
    // of their own
    std::vector<int32_t> cell_levels(n_cells, 0);
    std::vector<std::vector<int>> cell_width(n_cells);
    for (int g = 0; g < n_cells; g++) {
        if (cell_phys[g] < 0) continue;
        int a = m->phys_comp_off[cell_phys[g]], b = m->phys_comp_off[cell_phys[g] + 1];
        std::vector<int> dep(b - a, 0);
        int mx = 0;
        for (int i = 1; i < b - a; i++) {
            dep[i] = dep[m->comp_parent[a + i]] + 1;
            mx = std::max(mx, dep[i]);
        }
        cell_levels[g] = mx + 1;
        cell_width[g].assign(mx + 1, 0);
        for (int i = 0; i < b - a; i++) cell_width[g][dep[i]]++;
    }
    std::vector<int32_t> order(n_cells);
    std::iota(order.begin(), order.end(), 0);
    auto flagged = [&](int g) { return cell_phys[g] >= 0 && cell_f64[cell_phys[g]]; };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        bool ix = cell_phys[x] < 0, iy = cell_phys[y] < 0;
        if (ix != iy) return iy;  // physical cells first
        if (flagged(x) != flagged(y)) return flagged(y);
        if (cell_levels[x] != cell_levels[y]) return cell_levels[x] < cell_levels[y];
        return cell_n[x] < cell_n[y];
    });

    phase("units");
    // ---- units: each warp of the windowed kernel owns one unit for the whole
    // window -- a forest of physical cells (joint breadth-first numbering,
    // at most kForestWidth nodes per depth level, at most kForestNodes nodes) or a batch
    // of up to 32 izhikevich neurons.  Targets are numbered unit by unit.
    // Small networks get smaller forests, so that at least about four units
    // per SM run (a window's time is that of its slowest warp); large ones
    // fill forests up to kForestNodes.
    int forest_node_cap = kForestNodes;
    const int forest_width = (opt && opt->segments_per_depth > 0) ? std::min(opt->segments_per_depth, 1023) : kForestWidth;
    if (opt && opt->segments_per_warp > 0) {
        forest_node_cap = std::min(opt->segments_per_warp, 1023);
    } else {
        int64_t n_phys_comp = 0;
        int largest = 1;
        for (int k = 0; k < n_cells; k++)
            if (cell_phys[k] >= 0) {
                n_phys_comp += cell_n[k];
                largest = std::max(largest, cell_n[k]);
            }
        const int64_t units = 4 * (int64_t)std::max(ctx->n_sm, 1);
        const int64_t even = (n_phys_comp + units - 1) / units;
        forest_node_cap = (int)std::min<int64_t>(kForestNodes, std::max<int64_t>({even, (int64_t)largest, 8}));
    }
    std::vector<int32_t> u2i(nt, -1), i2u(nt, -1);
    std::vector<int32_t> c_parent(nt, -1), c_child0(nt, 0), c_nchild(nt, 0), t_izh(nt, -1);
    std::vector<float> c_u(nt, 0.f), c_l(nt, 0.f);
    std::vector<int32_t> fo_t0, fo_t1, fo_l0, fo_nlev, lvl;     // forests (also the per-step path's)
    std::vector<uint8_t> fo_f64;                                // forests solved in double precision
    std::vector<int32_t> un_t0, un_t1, un_f;                    // units: targets, forest or -1
    int next = 0;
    int max_forest = 1;
    int izh_slot = 0;
    std::vector<int32_t> izh_user_of_slot;
    {
        std::vector<int> phys, izhs;
        for (int k = 0; k < n_cells; k++) {
            if (cell_phys[order[k]] >= 0) phys.push_back(order[k]);
            else if (cell_izh[order[k]] >= 0) izhs.push_back(order[k]);
        }
        // the forests' cells, packed in schedule order
        std::vector<std::vector<int>> forests;
        size_t pi = 0;
        while (pi < phys.size()) {
            std::vector<int> fc;
            std::vector<int> fw;  // the forest's node count per depth
            int nodes = 0;
            while (pi < phys.size()) {
                const int c = phys[pi];
                const std::vector<int> &cw = cell_width[c];
                bool fits = fc.empty() || (nodes + cell_n[c] <= forest_node_cap && flagged(c) == flagged(fc.front()));
                for (size_t d = 0; fits && d < cw.size(); d++)
                    if ((d < fw.size() ? fw[d] : 0) + cw[d] > forest_width) fits = false;
                if (!fits && !fc.empty()) break;
                if (fw.size() < cw.size()) fw.resize(cw.size(), 0);
                for (size_t d = 0; d < cw.size(); d++) fw[d] += cw[d];
                fc.push_back(c);
                nodes += cell_n[c];
                pi++;
            }
            forests.push_back(std::move(fc));
        }
        // each forest's place: its first target and its depth boundaries
        // (a forest of depth D has D + 1 levels and D + 2 boundaries)
        const int nfo = (int)forests.size();
        fo_t0.resize(nfo); fo_t1.resize(nfo); fo_l0.resize(nfo); fo_nlev.resize(nfo); fo_f64.resize(nfo);
        for (int f = 0; f < nfo; f++) {
            int fn = 0, nl = 1;
            for (int g : forests[f]) { fn += cell_n[g]; nl = std::max(nl, (int)cell_levels[g]); }
            fo_t0[f] = next;
            fo_t1[f] = next + fn;
            fo_nlev[f] = nl;
            fo_l0[f] = (int)lvl.size();
            fo_f64[f] = flagged(forests[f].front()) ? 1 : 0;
            lvl.resize(lvl.size() + nl + 1);
            un_t0.push_back(next);
            un_f.push_back(f);
            next += fn;
            un_t1.push_back(next);
            max_forest = std::max(max_forest, fn);
        }
        // joint breadth-first numbering of each forest's cells, forests on
        // the host's threads (each writes only its own targets)
        parallel_for(nfo, [&](int64_t f) {
            const std::vector<int> &fc = forests[f];
            struct Node { int cell_base; int local; int depth; };
            std::vector<Node> q;
            std::vector<int> coff, kids, fill;
            for (int g : fc) q.push_back({m->phys_comp_off[cell_phys[g]], 0, 0});
            const int f_t0 = fo_t0[f];
            int32_t *lv = &lvl[fo_l0[f]];
            lv[0] = f_t0;
            int depth = 0;
            std::vector<std::vector<int>> cell_kids(fc.size());
            for (size_t ci = 0; ci < fc.size(); ci++) {
                const int pcell = cell_phys[fc[ci]];
                const int a0 = m->phys_comp_off[pcell], n0 = m->phys_comp_off[pcell + 1] - a0;
                coff.assign(n0 + 1, 0);
                for (int i = 1; i < n0; i++) coff[m->comp_parent[a0 + i] + 1]++;
                for (int i = 0; i < n0; i++) coff[i + 1] += coff[i];
                kids.assign(n0 > 1 ? n0 - 1 : 1, 0);
                fill.assign(n0, 0);
                for (int i = 1; i < n0; i++) {
                    const int pp = m->comp_parent[a0 + i];
                    kids[coff[pp] + fill[pp]++] = i;
                }
                std::vector<int> &ck = cell_kids[ci];  // [coff (n0+1)] [kids (n0-1)]
                ck.assign(coff.begin(), coff.end());
                ck.insert(ck.end(), kids.begin(), kids.begin() + std::max(0, n0 - 1));
            }
            std::vector<int> node_cell;
            for (size_t ci = 0; ci < fc.size(); ci++) node_cell.push_back((int)ci);
            for (size_t h = 0; h < q.size(); h++) {
                const Node u = q[h];
                const int ci = node_cell[h];
                if (u.depth != depth) {
                    depth = u.depth;
                    lv[depth] = f_t0 + (int)h;
                }
                const int it = f_t0 + (int)h;
                const int ut = u.cell_base + u.local;
                u2i[ut] = it;
                i2u[it] = ut;
                const std::vector<int> &ck = cell_kids[ci];
                const int pcell = cell_phys[fc[ci]];
                const int n0 = m->phys_comp_off[pcell + 1] - m->phys_comp_off[pcell];
                const int k0 = ck[u.local], k1 = ck[u.local + 1];
                c_nchild[it] = k1 - k0;
                c_child0[it] = k1 > k0 ? f_t0 + (int)q.size() : 0;
                for (int k = k0; k < k1; k++) {
                    q.push_back({u.cell_base, ck[n0 + 1 + k], u.depth + 1});
                    node_cell.push_back(ci);
                }
            }
            lv[fo_nlev[f]] = f_t0 + (int)q.size();
        }, 32);
        for (size_t k = 0; k < izhs.size(); k += 32) {
            un_t0.push_back(next);
            un_f.push_back(-1);
            for (size_t j = k; j < std::min(izhs.size(), k + 32); j++) {
                const int ut = n_comp + cell_izh[izhs[j]];
                u2i[ut] = next;
                i2u[next] = ut;
                t_izh[next] = izh_slot++;
                izh_user_of_slot.push_back(cell_izh[izhs[j]]);
                next++;
            }
            un_t1.push_back(next);
        }
    }
    if (next != nt) return ctx->fail(EDEN_GPU_E_INVALID, "cells not covered by spike sources");
    // parents and off-diagonals in internal numbering
    for (int it = 0; it < nt; it++) {
        int ut = i2u[it];
        if (ut >= n_comp) continue;
        int pcell = comp_cell[ut];
        int a = m->phys_comp_off[pcell];
        int p = m->comp_parent[ut];
        if (p >= 0) {
            c_parent[it] = u2i[a + p];
            float R = m->comp_r_axial[ut];
            c_u[it] = -dt / (R * m->comp_c[ut]);
            c_l[it] = -dt / (R * m->comp_c[a + p]);
        }
    }
    // end of each node's child range (children of consecutive nodes are consecutive)
    std::vector<int32_t> c_cend(nt, 0);
    for (int it = 0; it < nt; it++) c_cend[it] = c_child0[it] + c_nchild[it];
    for (size_t f = 0; f < fo_t0.size(); f++) {
        // nodes without children still need the running end for their successor
        int run = lvl[fo_l0[f] + 1 < (int)lvl.size() ? fo_l0[f] + 1 : fo_l0[f]];
        if (fo_nlev[f] == 1) run = fo_t1[f];
        for (int it = fo_t0[f]; it < fo_t1[f]; it++) {
            if (c_nchild[it] > 0) run = c_child0[it] + c_nchild[it];
            c_cend[it] = run;
        }
    }
    ctx->user_to_internal = u2i;
    ctx->gcap = max_cell;
    ctx->forest_cap = max_forest;
    phase("constants");
    // ---- per-target constants in internal order
    std::vector<float> c_cm(nt, 1.f), c_inv(nt, 0.f), c_area(nt, 0.f), v0(nt, 0.f);
    std::vector<int32_t> c_chan0(nt + 1, 0);
    parallel_for(nt, [&](int64_t it) {
        int ut = i2u[it];
        if (ut < n_comp) {
            c_cm[it] = m->comp_c[ut];
            c_inv[it] = m->comp_inv_rc[ut];
            c_area[it] = m->comp_area[ut];
            v0[it] = m->comp_v0[ut];
            c_chan0[it + 1] = m->comp_chan_off[ut + 1] - m->comp_chan_off[ut];
        } else {
            // the value the initialisation passes give V (OnStart)
            const int64_t uk = ut - n_comp;
            const int kind = m->izh_kind ? m->izh_kind[uk] : EDEN_POINT_IZH2007;
            const int f = kind == EDEN_POINT_FN ? 1
                          : kind == EDEN_POINT_IZH2007 ? 1
                          : (kind == EDEN_POINT_IAF_TAU || kind == EDEN_POINT_IAF_TAU_REF || kind == EDEN_POINT_IZH_DL) ? 0
                                                                                                                   : 2;
            v0[it] = m->izh_params[EDEN_POINT_PARAMS * uk + f];
        }
    });
    for (int it = 0; it < nt; it++) c_chan0[it + 1] += c_chan0[it];
    int n_chan = c_chan0[nt];
    std::vector<int32_t> ch_type(n_chan), ch_gate0(n_chan + 1, 0);
    std::vector<float> ch_g(n_chan), ch_e(n_chan);
    parallel_for(nt, [&](int64_t it) {
        int ut = i2u[it];
        if (ut >= n_comp) return;
        int o = c_chan0[it];
        for (int ch = m->comp_chan_off[ut]; ch < m->comp_chan_off[ut + 1]; ch++, o++) {
            ch_type[o] = m->chan_type[ch];
            ch_g[o] = m->chan_gbase[ch];
            ch_e[o] = m->chan_erev[ch];
        }
    });
    for (int ch = 0; ch < n_chan; ch++) ch_gate0[ch + 1] = ch_gate0[ch] + m->chan_types[ch_type[ch]].n_gates;
    int n_gate = ch_gate0[n_chan];

    // flat parameters of compartments with one gateless channel and no inputs
    std::vector<float> flat_g(nt, -1.0f), flat_e(nt, 0.f), flat_gc(nt, 0.f), flat_d0(nt, 0.f);
    {
        std::vector<char> has_input(nt, 0);
        for (int64_t k = 0; k < m->n_pulse; k++) has_input[u2i[m->pulse_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_pois; k++) has_input[u2i[m->pois_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_syn; k++) has_input[u2i[m->syn_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_timed; k++) has_input[u2i[m->timed_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_wave; k++) has_input[u2i[m->wave_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_clamp; k++) has_input[u2i[m->clamp_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_gap; k++) has_input[u2i[m->gap_target[k]]] = 1;
        for (int64_t k = 0; k < m->n_graded; k++) has_input[u2i[m->graded_target[k]]] = 1;
        parallel_for(nt, [&](int64_t it) {
            if (t_izh[it] >= 0 || has_input[it]) return;
            if (c_chan0[it + 1] - c_chan0[it] != 1) return;
            const int ch = c_chan0[it];
            if (m->chan_types[ch_type[ch]].n_gates != 0) return;
            const float g = ch_g[ch];
            if (!(g >= 0.0f)) return;
            // the same operations as the general path with fopen = 1 and no inputs
            const float gs = g * 1.0f;
            const float Gc = (gs * 1e-5f) * c_area[it];
            const float G = Gc + 0.0f + 0.0f;
            flat_g[it] = gs;
            flat_e[it] = ch_e[ch];
            flat_gc[it] = G;
            flat_d0[it] = 1.0f * (G / c_cm[it]) + c_inv[it];
        });
    }

    // windowed-path constants (see DevModel::c_kl): a compartment is flat when
    // it has one gateless channel and no inputs, is no spike source, and every
    // compartment below it is flat; its pivot and elimination factor are then
    // the same every step and are computed here once, deepest first
    std::vector<char> nonflat(nt, 1);
    std::vector<float> c_kc(nt, 0.f), c_pv0(nt, 0.f), c_rt0(nt, 0.f);
    std::vector<uint32_t> c_cep(nt, 0);
    {
        std::vector<char> is_src(nt, 0);
        for (int s = 0; s < m->n_src; s++)
            if (m->src_target[s] >= 0) is_src[u2i[m->src_target[s]]] = 1;
        // (forests on the host's threads; each writes its own compartments)
        parallel_for((int64_t)fo_t0.size(), [&](int64_t f) {
            const int a = fo_t0[f], b = fo_t1[f];
            for (int it = b - 1; it >= a; it--) {
                const int k0 = c_child0[it], k1 = c_child0[it] + c_nchild[it];
                bool flat = flat_g[it] >= 0.0f && !is_src[it];
                for (int c = k0; flat && c < k1; c++) flat = !nonflat[c];
                nonflat[it] = flat ? 0 : 1;
                if (flat) {
                    c_kc[it] = (dt * (flat_gc[it] * flat_e[it])) / c_cm[it];
                    float dj = 1.0f + flat_d0[it] * dt;
                    for (int c = k0; c < k1; c++) dj -= c_rt0[c] * c_u[c];
                    const float inv = 1.0f / dj;
                    c_pv0[it] = inv;
                    c_rt0[it] = c_l[it] * inv;
                }
                const uint32_t cb = k1 > k0 ? (uint32_t)(k0 - a) : 0u, ce = k1 > k0 ? (uint32_t)(k1 - a) : 0u;
                const uint32_t pp = c_parent[it] >= 0 ? (uint32_t)(c_parent[it] - a + 1) : 0u;
                c_cep[it] = ce | (cb << kCepBeginShift) | (pp << kCepParentShift) | (nonflat[it] ? kCepNonFlat : 0u);
            }
        }, 32);
    }
    // a flat compartment's pre-update increment, or a non-flat one's L
    std::vector<float> c_kl(nt, 0.f);
    for (int it = 0; it < nt; it++) c_kl[it] = nonflat[it] ? c_l[it] : c_kc[it];

    // per forest depth (parallel to lvl): non-flat flag
    std::vector<uint8_t> lvl_info(lvl.size(), 0);
    for (size_t f = 0; f < fo_t0.size(); f++)
        for (int l = 0; l < fo_nlev[f]; l++)
            for (int it = lvl[fo_l0[f] + l]; it < lvl[fo_l0[f] + l + 1]; it++)
                if (nonflat[it]) lvl_info[fo_l0[f] + l] = 0x80;
    // gate parameter records per channel type and gate (gate_next_p)
    std::vector<float> gate_par((size_t)std::max(m->n_chan_types, 1) * EDEN_MAX_GATES * kGateWords, 0.f);
    for (int k = 0; k < m->n_chan_types; k++) {
        const EdenGpuChannelType &ty = m->chan_types[k];
        for (int g = 0; g < ty.n_gates; g++) {
            float *r = &gate_par[((size_t)k * EDEN_MAX_GATES + g) * kGateWords];
            int32_t fk = ty.fwd_kind[g], rk = ty.rev_kind[g];
            if (ty.gate_kind[g] != EDEN_GATE_RATES) fk |= (1 + k * EDEN_MAX_GATES + g) << 8;
            memcpy(&r[0], &fk, 4); r[1] = ty.fwd_rate[g]; r[2] = ty.fwd_mid[g]; r[3] = ty.fwd_scale[g];
            memcpy(&r[4], &rk, 4); r[5] = ty.rev_rate[g]; r[6] = ty.rev_mid[g]; r[7] = ty.rev_scale[g];
            r[8] = ty.q10[g];
        }
    }

    // kinds and timeCourse / steadyState forms of the gates of other kinds
    // than gateHHrates, by channel type and gate (gate_next_p)
    std::vector<float> gate_ext((size_t)std::max(m->n_chan_types, 1) * EDEN_MAX_GATES * kGateExtWords, 0.f);
    bool gate_forms = false;
    for (int k = 0; k < m->n_chan_types; k++) {
        const EdenGpuChannelType &ty = m->chan_types[k];
        for (int g = 0; g < ty.n_gates; g++) {
            float *r = &gate_ext[((size_t)k * EDEN_MAX_GATES + g) * kGateExtWords];
            int32_t gk = ty.gate_kind[g], tk = ty.tau_kind[g], ik = ty.inf_kind[g];
            gate_forms |= gk != EDEN_GATE_RATES;
            memcpy(&r[0], &gk, 4);
            memcpy(&r[1], &tk, 4); r[2] = ty.tau_rate[g]; r[3] = ty.tau_mid[g]; r[4] = ty.tau_scale[g];
            memcpy(&r[5], &ik, 4); r[6] = ty.inf_rate[g]; r[7] = ty.inf_mid[g]; r[8] = ty.inf_scale[g];
        }
    }

    // point neurons: kinds and parameters (field-major) in slot (internal) order
    std::vector<int32_t> iz_kind(n_izh);
    std::vector<float> iz_p((size_t)EDEN_POINT_PARAMS * std::max(n_izh, 1), 0.0f);
    for (int k = 0; k < n_izh; k++) {
        const int64_t uk = izh_user_of_slot[k];
        iz_kind[k] = m->izh_kind ? m->izh_kind[uk] : EDEN_POINT_IZH2007;
        for (int f = 0; f < EDEN_POINT_PARAMS; f++)
            iz_p[(size_t)f * n_izh + k] = m->izh_params[EDEN_POINT_PARAMS * uk + f];
    }

    phase("inputs-sort");
    // ---- inputs sorted by internal target (then type, then input order)
    // (two stable counting passes: by type, then by internal target)
    auto sort_items = [&](int64_t n, const int32_t *tgt, const int32_t *type) {
        std::vector<int64_t> idx(n), tmp(n);
        std::iota(idx.begin(), idx.end(), 0);
        // each item's internal target, looked up once (on the host's threads)
        std::vector<int32_t> tkey(n);
        parallel_for(n, [&](int64_t x) { tkey[x] = u2i[tgt[x]]; });
        auto pass = [&](int nkeys, auto key) {
            std::vector<int64_t> cnt((size_t)nkeys + 1, 0);
            for (int64_t k = 0; k < n; k++) cnt[key(idx[k]) + 1]++;
            for (int b = 0; b < nkeys; b++) cnt[b + 1] += cnt[b];
            for (int64_t k = 0; k < n; k++) tmp[cnt[key(idx[k])]++] = idx[k];
            idx.swap(tmp);
        };
        // (the pass by type only where the items have more than one)
        bool one_type = true;
        for (int64_t x = 1; type && one_type && x < n; x++) one_type = type[x] == type[0];
        if (type && !one_type) pass(kMaxSynTypes, [&](int64_t x) { return (int)type[x]; });
        pass(nt, [&](int64_t x) { return (int)tkey[x]; });
        return idx;
    };
    auto offsets = [&](const std::vector<int64_t> &order, const int32_t *tgt) {
        std::vector<int64_t> off(nt + 1, 0);
        for (int64_t k : order) off[u2i[tgt[k]] + 1]++;
        for (int t = 0; t < nt; t++) off[t + 1] += off[t];
        return off;
    };
    // (the Poisson inputs and the synapses, the two large sets, sort side by side)
    std::vector<int64_t> qord = sort_items(m->n_pulse, m->pulse_target, nullptr), pord, sord;
    {
        std::thread tp([&] { pord = sort_items(m->n_pois, m->pois_target, m->pois_type); });
        sord = sort_items(m->n_syn, m->syn_target, m->syn_type);
        tp.join();
    }
    std::vector<int64_t> qoff = offsets(qord, m->pulse_target);
    std::vector<int64_t> poff = offsets(pord, m->pois_target);
    std::vector<int64_t> soff = offsets(sord, m->syn_target);
    std::vector<float> pu_s(m->n_pulse), pu_d(m->n_pulse), pu_a(m->n_pulse), pu_w(m->n_pulse);
    for (int64_t k = 0; k < m->n_pulse; k++) {
        int64_t o = qord[k];
        pu_s[k] = m->pulse_start[o]; pu_d[k] = m->pulse_duration[o];
        pu_a[k] = m->pulse_amplitude[o]; pu_w[k] = m->pulse_weight[o];
    }
    // sine / ramp generators by internal target, then shape (input order within a shape)
    std::vector<int64_t> word = sort_items(m->n_wave, m->wave_target, m->wave_shape);
    std::vector<int64_t> woff = offsets(word, m->wave_target);
    std::vector<float> wv_p((size_t)m->n_wave * kWaveWords, 0.f);
    std::vector<uint8_t> wv_shape(m->n_wave);
    for (int64_t k = 0; k < m->n_wave; k++) {
        const int64_t o = word[k];
        for (int j = 0; j < EDEN_WAVE_PARAMS; j++) wv_p[k * kWaveWords + j] = m->wave_params[EDEN_WAVE_PARAMS * o + j];
        wv_p[k * kWaveWords + EDEN_WAVE_PARAMS] = m->wave_weight[o];
        wv_shape[k] = (uint8_t)m->wave_shape[o];
    }
    // voltage clamps by internal target (input order within a target)
    std::vector<int64_t> clord = sort_items(m->n_clamp, m->clamp_target, nullptr);
    std::vector<int64_t> cloff = offsets(clord, m->clamp_target);
    std::vector<float> cl_p((size_t)m->n_clamp * kClampWords, 0.f);
    for (int64_t k = 0; k < m->n_clamp; k++) {
        const int64_t o = clord[k];
        for (int j = 0; j < EDEN_CLAMP_PARAMS; j++) cl_p[k * kClampWords + j] = m->clamp_params[EDEN_CLAMP_PARAMS * o + j];
        cl_p[k * kClampWords + EDEN_CLAMP_PARAMS] = m->clamp_weight[o];
    }
    std::vector<float> po_rate(m->n_pois), po_w(m->n_pois);
    std::vector<int32_t> po_seed(m->n_pois), po_inst(m->n_pois), po_rng(m->n_pois);
    std::vector<uint8_t> po_type(m->n_pois);
    parallel_for(m->n_pois, [&](int64_t k) {
        int64_t o = pord[k];
        po_rate[k] = m->pois_rate[o]; po_w[k] = m->pois_weight[o];
        po_seed[k] = m->src_cell_seed[m->pois_src[o]];
        po_inst[k] = m->pois_instance[o];
        po_rng[k] = m->pois_rng_base ? m->pois_rng_base[o] : 0;
        po_type[k] = (uint8_t)m->pois_type[o];
    });
    // timedSynapticInput items sorted by internal target (then type, then input order)
    std::vector<int64_t> tord = sort_items(m->n_timed, m->timed_target, m->timed_type);
    std::vector<int64_t> toff = offsets(tord, m->timed_target);
    std::vector<float> tm_w(m->n_timed);
    std::vector<uint8_t> tm_type(m->n_timed);
    std::vector<int64_t> tm_off(m->n_timed + 1, 0), tm_step;
    for (int64_t k = 0; k < m->n_timed; k++) {
        const int64_t o = tord[k];
        tm_w[k] = m->timed_weight[o];
        tm_type[k] = (uint8_t)m->timed_type[o];
        tm_step.insert(tm_step.end(), m->timed_step + m->timed_off[o], m->timed_step + m->timed_off[o + 1]);
        tm_off[k + 1] = (int64_t)tm_step.size();
    }
    const int64_t ns = m->n_syn;
    ctx->n_syn = ns;
    std::vector<float> sy_w(ns), sy_d(ns), sy_pend(ns, -INFINITY);
    std::vector<uint8_t> sy_type(ns);
    ctx->syn_internal_of_user.assign(ns, 0);
    float min_delay = INFINITY;
    parallel_for(ns, [&](int64_t k) {
        int64_t o = sord[k];
        sy_w[k] = m->syn_weight[o]; sy_d[k] = m->syn_delay[o];
        sy_type[k] = (uint8_t)m->syn_type[o];
        ctx->syn_internal_of_user[o] = k;
    });
    for (int64_t k = 0; k < ns; k++) min_delay = std::min(min_delay, m->syn_delay[k]);
    phase("fanout");
    // source fan-out in connection (user) order
    std::vector<int64_t> fan0(m->n_src + 1, 0);
    for (int64_t o = 0; o < ns; o++) fan0[m->syn_src[o] + 1]++;
    for (int s = 0; s < m->n_src; s++) fan0[s + 1] += fan0[s];
    std::vector<int32_t> fan_syn(ns);
    {
        std::vector<int64_t> fill(m->n_src, 0);
        for (int64_t o = 0; o < ns; o++) {
            int s = m->syn_src[o];
            fan_syn[fan0[s] + fill[s]++] = (int32_t)ctx->syn_internal_of_user[o];
        }
    }
    std::vector<int32_t> t_src(nt, -1);
    std::vector<float> src_thr(m->n_src);
    for (int s = 0; s < m->n_src; s++) {
        if (m->src_target[s] >= 0) t_src[u2i[m->src_target[s]]] = s;
        src_thr[s] = m->src_threshold[s];
    }
    phase("blocks");
    // input blocks per target: pulses, then Poisson runs, timed-input runs, then synapse runs of one type
    std::vector<int32_t> t_blk0(nt + 1, 0);
    std::vector<int32_t> bk_kind;
    std::vector<uint8_t> bk_type;
    std::vector<float> bk_erev;
    std::vector<int64_t> bk_i0, bk_i1;
    std::vector<int32_t> in_tgt;
    for (int t = 0; t < nt; t++) {
        t_blk0[t] = (int32_t)bk_kind.size();
        if (qoff[t + 1] > qoff[t]) {
            bk_kind.push_back(BK_PULSE); bk_erev.push_back(0.f); bk_type.push_back(0);
            bk_i0.push_back(qoff[t]); bk_i1.push_back(qoff[t + 1]);
        }
        if (cloff[t + 1] > cloff[t]) {
            bk_kind.push_back(BK_PULSE); bk_erev.push_back(0.f); bk_type.push_back((uint8_t)kClampA);
            bk_i0.push_back(cloff[t]); bk_i1.push_back(cloff[t + 1]);
            bk_kind.push_back(BK_CLAMPV); bk_erev.push_back(0.f); bk_type.push_back((uint8_t)kClampB);
            bk_i0.push_back(cloff[t]); bk_i1.push_back(cloff[t + 1]);
        }
        for (int64_t k = woff[t]; k < woff[t + 1];) {
            int64_t k1 = k;
            while (k1 < woff[t + 1] && wv_shape[k1] == wv_shape[k]) k1++;
            bk_kind.push_back(BK_PULSE); bk_erev.push_back(0.f); bk_type.push_back((uint8_t)(1 + wv_shape[k]));
            bk_i0.push_back(k); bk_i1.push_back(k1);
            k = k1;
        }
        for (int64_t k = poff[t]; k < poff[t + 1];) {
            int64_t k1 = k;
            while (k1 < poff[t + 1] && po_type[k1] == po_type[k]) k1++;
            bk_kind.push_back(BK_POIS | (current_kind(m->syn_types[po_type[k]].kind) ? BK_CURRENT : 0));
            bk_erev.push_back(m->syn_types[po_type[k]].erev); bk_type.push_back(po_type[k]);
            bk_i0.push_back(k); bk_i1.push_back(k1);
            k = k1;
        }
        for (int64_t k = toff[t]; k < toff[t + 1];) {
            int64_t k1 = k;
            while (k1 < toff[t + 1] && tm_type[k1] == tm_type[k]) k1++;
            bk_kind.push_back(BK_TIMED | (current_kind(m->syn_types[tm_type[k]].kind) ? BK_CURRENT : 0));
            bk_erev.push_back(m->syn_types[tm_type[k]].erev); bk_type.push_back(tm_type[k]);
            bk_i0.push_back(k); bk_i1.push_back(k1);
            k = k1;
        }
        for (int64_t k = soff[t]; k < soff[t + 1];) {
            int64_t k1 = k;
            while (k1 < soff[t + 1] && sy_type[k1] == sy_type[k]) k1++;
            const EdenGpuSynapseType &sk = m->syn_types[sy_type[k]];
            const bool blocked = sk.kind == EDEN_SYN_BLOCKING_PLASTIC && sk.block_volt != 0.0f;
            bk_kind.push_back(BK_SYN | (current_kind(sk.kind) ? BK_CURRENT : 0) | (blocked ? BK_BLOCK : 0));
            bk_erev.push_back(sk.erev); bk_type.push_back(sy_type[k]);
            bk_i0.push_back(k); bk_i1.push_back(k1);
            k = k1;
        }
        if ((int)bk_kind.size() > t_blk0[t]) in_tgt.push_back(t);
    }
    t_blk0[nt] = (int32_t)bk_kind.size();
    const int n_block = (int)bk_kind.size();
    // chunks of at most kChunkItems items per block
    std::vector<int32_t> bk_c0(n_block + 1, 0), ck_blk, ck_n;
    std::vector<int64_t> ck_i0;
    for (int b = 0; b < n_block; b++) {
        bk_c0[b] = (int32_t)ck_blk.size();
        for (int64_t i = bk_i0[b]; i < bk_i1[b]; i += kChunkItems) {
            ck_blk.push_back(b);
            ck_i0.push_back(i);
            ck_n.push_back((int32_t)std::min<int64_t>(kChunkItems, bk_i1[b] - i));
        }
    }
    bk_c0[n_block] = (int32_t)ck_blk.size();
    const int n_chunk = (int)ck_blk.size();
    std::vector<int32_t> ck_info(n_chunk);
    for (int c = 0; c < n_chunk; c++)
        ck_info[c] = (bk_kind[ck_blk[c]] == BK_CLAMPV ? BK_PULSE : (bk_kind[ck_blk[c]] & BK_KIND_MASK)) |
                     ((int32_t)bk_type[ck_blk[c]] << 2) | (ck_n[c] << 8);

    // ---- window length: every delay must cover the window (see k_window)
    int kmax = kMaxWindow;
    if (ns > 0) {
        double dsteps = std::floor((double)min_delay / (double)dt);
        kmax = (int)std::max(1.0, std::min((double)kMaxWindow, dsteps));
    }
    // gap junctions couple cells within a step: one-step windows, each
    // reading its peers' potentials from the buffer the previous one wrote
    if (m->n_gap > 0 || m->n_graded > 0) kmax = 1;
    ctx->mode = opt ? opt->mode : EDEN_MODE_PLAIN;
    ctx->kernel_timing = opt && opt->kernel_timing;
    int kreq = (opt && opt->steps_per_launch > 0) ? opt->steps_per_launch : kmax;
    ctx->K = ctx->mode == EDEN_MODE_BATCHED ? std::max(1, std::min(kreq, kmax)) : 1;

    // ---- recording
    // each column on its target's list, with the internal gate slot it
    // records or -1 for the membrane potential
    int32_t n_trace = opt ? opt->n_trace : 0;
    std::vector<int32_t> t_trace0(nt + 1, 0), trace_col(n_trace), trace_gate(n_trace, -1);
    {
        std::vector<int64_t> ugate0(m->comp_chan_off[n_comp] + 1, 0);  // user gate numbering
        for (int32_t ch = 0; ch < m->comp_chan_off[n_comp]; ch++)
            ugate0[ch + 1] = ugate0[ch] + m->chan_types[m->chan_type[ch]].n_gates;
        std::vector<std::vector<std::pair<int, int>>> cols(nt);
        for (int j = 0; j < n_trace; j++) {
            const int32_t code = opt->trace_target[j];
            if (code >= 0) {
                if (code >= nt) return ctx->fail(EDEN_GPU_E_INVALID, "trace column %d: bad target", j);
                cols[u2i[code]].push_back({j, -1});
                continue;
            }
            const int64_t g = -2 - (int64_t)code;
            if (code == -1 || g >= ugate0.back())
                return ctx->fail(EDEN_GPU_E_INVALID, "trace column %d: bad gate", j);
            const int32_t ch = (int32_t)(std::upper_bound(ugate0.begin(), ugate0.end(), g) - ugate0.begin()) - 1;
            const int32_t comp = (int32_t)(std::upper_bound(m->comp_chan_off, m->comp_chan_off + n_comp + 1, ch) -
                                           m->comp_chan_off) - 1;
            const int it = u2i[comp];
            const int o = c_chan0[it] + (ch - m->comp_chan_off[comp]);
            cols[it].push_back({j, ch_gate0[o] + (int)(g - ugate0[ch])});
        }
        for (int t = 0; t < nt; t++) t_trace0[t + 1] = t_trace0[t] + (int)cols[t].size();
        for (int t = 0; t < nt; t++)
            for (size_t k = 0; k < cols[t].size(); k++) {
                trace_col[t_trace0[t] + k] = cols[t][k].first;
                trace_gate[t_trace0[t] + k] = cols[t][k].second;
            }
    }
    ctx->n_trace = n_trace;
    ctx->trace_cap = (opt && opt->record_capacity_steps > 0) ? opt->record_capacity_steps : 4096;
    int64_t log_cap = (opt && opt->spike_capacity > 0) ? opt->spike_capacity : (int64_t)1 << 22;

    phase("unit-lists");
    // ---- per-unit lists of the windowed kernel: spike sources and recorded
    // targets (unit-local indices), gates, and each unit's shared-memory words
    const int n_unit = (int)un_t0.size();
    std::vector<int32_t> un_gt0(n_unit), un_ngt(n_unit), un_s0(n_unit), un_s1(n_unit), un_r0(n_unit), un_r1(n_unit);
    std::vector<int32_t> gs_t, gs_src, gr_t, gr_col;
    std::vector<float> gs_thr;
    std::vector<int32_t> un_nf0(n_unit), un_nf1(n_unit), nf_t;
    std::vector<int> un_words(n_unit);
    {
        std::vector<int32_t> slot_of(nt, -1);
        for (int u = 0; u < n_unit; u++) {
            const int a = un_t0[u], b = un_t1[u];
            un_nf0[u] = (int)nf_t.size();
            if (un_f[u] >= 0)
                for (int t = a; t < b; t++)
                    if (nonflat[t]) { slot_of[t] = (int)nf_t.size() - un_nf0[u]; nf_t.push_back(t - a); }
            un_nf1[u] = (int)nf_t.size();
        }
        for (int u = 0; u < n_unit; u++) {
            const int a = un_t0[u], b = un_t1[u];
            un_s0[u] = (int)gs_t.size();
            if (un_f[u] >= 0)
                for (int t = a; t < b; t++)
                    if (t_src[t] >= 0) { gs_t.push_back(slot_of[t]); gs_src.push_back(t_src[t]); gs_thr.push_back(src_thr[t_src[t]]); }
            un_s1[u] = (int)gs_t.size();
        }
    }
    // channels of each unit's non-flat compartments, in slot order, and the
    // channel set of each (the generated code has one routine per set)
    std::vector<int32_t> nf_c0(nf_t.size()), nf_c1(nf_t.size()), nfc_q, nfc_i, nf_sig(nf_t.size(), -1);
    std::map<std::vector<int>, int> set_id;
    std::vector<std::vector<int>> chan_sets;
    std::vector<float> nfc_g, nfc_e;
    for (int u = 0; u < n_unit; u++) {
        const int a = un_t0[u];
        const int gbase = ch_gate0[c_chan0[a]];
        for (int k = un_nf0[u]; k < un_nf1[u]; k++) {
            const int t = a + nf_t[k];
            nf_c0[k] = (int)nfc_g.size();
            std::vector<int> set;
            for (int ch = c_chan0[t]; ch < c_chan0[t + 1]; ch++) set.push_back(ch_type[ch]);
            auto found = set_id.find(set);
            if (found != set_id.end()) {
                nf_sig[k] = found->second;
            } else if (chan_sets.size() < 64) {
                nf_sig[k] = (int)chan_sets.size();
                set_id[set] = nf_sig[k];
                chan_sets.push_back(set);
            }
            for (int ch = c_chan0[t]; ch < c_chan0[t + 1]; ch++) {
                const EdenGpuChannelType &ty = m->chan_types[ch_type[ch]];
                int32_t pack = ty.n_gates;
                for (int g = 0; g < ty.n_gates; g++) pack |= ty.gate_instances[g] << (3 + 5 * g);
                nfc_g.push_back(ch_g[ch]); nfc_e.push_back(ch_e[ch]);
                nfc_q.push_back(ch_gate0[ch] - gbase); nfc_i.push_back(pack);
            }
            nf_c1[k] = (int)nfc_g.size();
        }
    }
    for (int u = 0; u < n_unit; u++) {
        const int a = un_t0[u], b = un_t1[u];
        un_gt0[u] = ch_gate0[c_chan0[a]];
        // a unit's trace columns: its local target, or -1 - its local gate slot
        un_r0[u] = (int)gr_t.size();
        for (int t = a; t < b; t++)
            for (int k = t_trace0[t]; k < t_trace0[t + 1]; k++) {
                gr_t.push_back(trace_gate[k] < 0 ? t - a : -1 - (trace_gate[k] - un_gt0[u]));
                gr_col.push_back(trace_col[k]);
            }
        un_r1[u] = (int)gr_t.size();
        un_ngt[u] = ch_gate0[c_chan0[b]] - un_gt0[u];
        if (un_f[u] >= 0) {
            const int nblk = t_blk0[b] - t_blk0[a];
            const int nck = bk_c0[t_blk0[b]] - bk_c0[t_blk0[a]];
            const int nfch = un_nf1[u] > un_nf0[u] ? nf_c1[un_nf1[u] - 1] - nf_c0[un_nf0[u]] : 0;
            un_words[u] = forest_words(b - a, un_nf1[u] - un_nf0[u], nfch, un_ngt[u], fo_nlev[un_f[u]],
                                       un_s1[u] - un_s0[u], nblk, nck, std::max(ctx->K, 4), fo_f64[un_f[u]] != 0);
        } else {
            un_words[u] = izh_words(b - a);
        }
    }
    phase("packing");
    // CTAs of up to four units, packed longest-first onto the CTA with the
    // fewest words so that every CTA needs about the same shared memory; a
    // network of more CTAs than SMs gets a multiple of the SM count of them
    // (some then hold three units), so that every SM runs as many (1 % faster
    // on C2).  (Packing by an estimate of each unit's work instead measured
    // 3 % slower.)
    const int upc = kCellThreads / 32;
    int n_cta = (n_unit + upc - 1) / upc;
    if (n_cta > ctx->n_sm) n_cta = std::min(n_unit, (n_cta + ctx->n_sm - 1) / ctx->n_sm * ctx->n_sm);
    std::vector<int> uorder(n_unit);
    std::iota(uorder.begin(), uorder.end(), 0);
    std::stable_sort(uorder.begin(), uorder.end(), [&](int x, int y) { return un_words[x] > un_words[y]; });
    std::vector<std::vector<int>> cta_units(n_cta);
    std::vector<int> cta_words(n_cta, 0);
    {
        // min-heap of (words, cta) over CTAs that still have room
        std::vector<std::pair<int, int>> heap;
        for (int c = 0; c < n_cta; c++) heap.push_back({0, c});
        auto cmp = [](const std::pair<int, int> &x, const std::pair<int, int> &y) { return x > y; };
        std::make_heap(heap.begin(), heap.end(), cmp);
        for (int uu : uorder) {
            std::pop_heap(heap.begin(), heap.end(), cmp);
            auto top = heap.back();
            heap.pop_back();
            cta_units[top.second].push_back(uu);
            cta_words[top.second] += un_words[uu];
            if ((int)cta_units[top.second].size() < upc) {
                heap.push_back({cta_words[top.second], top.second});
                std::push_heap(heap.begin(), heap.end(), cmp);
            }
        }
    }
    std::vector<int32_t> cta_u0, un_off(n_unit, 0), unit_of_slot;
    for (int c = 0; c < n_cta; c++) {
        cta_u0.push_back((int)unit_of_slot.size());
        for (int uu : cta_units[c]) unit_of_slot.push_back(uu);
    }
    cta_u0.push_back((int)unit_of_slot.size());
    // units are referenced through their CTA slot: renumber the unit tables in slot order
    auto perm = [&](std::vector<int32_t> &v) {
        std::vector<int32_t> o(v.size());
        for (size_t j = 0; j < unit_of_slot.size(); j++) o[j] = v[unit_of_slot[j]];
        v.swap(o);
    };
    for (auto *v : {&un_t0, &un_t1, &un_f, &un_gt0, &un_ngt, &un_s0, &un_s1, &un_r0, &un_r1, &un_nf0, &un_nf1}) perm(*v);
    {
        std::vector<int> w2(n_unit);
        for (int j = 0; j < n_unit; j++) w2[j] = un_words[unit_of_slot[j]];
        un_words.swap(w2);
    }
    for (size_t c = 0; c + 1 < cta_u0.size(); c++) {
        int off = 0;
        for (int j = cta_u0[c]; j < cta_u0[c + 1]; j++) { un_off[j] = off; off += un_words[j]; }
    }
    // one launch over all CTAs, sized by the largest
    ctx->classes.clear();
    {
        int mx = 1;
        for (int c = 0; c < n_cta; c++) mx = std::max(mx, cta_words[c]);
        ctx->classes.push_back({0, n_cta, (size_t)mx * sizeof(float)});
    }
    size_t max_smem_class = 0;
    for (auto &cl : ctx->classes) max_smem_class = std::max(max_smem_class, cl.smem);
    // (the windowed kernel packs forest-local indices in 10 bits: a single
    // cell of more than 1023 compartments runs the per-step kernels)
    // (the forward-Euler update runs the per-step kernels only)
    // (and a model with blockingPlasticSynapses, whose voltage block the
    // per-step kernels apply)
    bool plastic_syn = false;
    for (int k = 0; k < m->n_syn_types; k++) plastic_syn |= m->syn_types[k].kind == EDEN_SYN_BLOCKING_PLASTIC;
    ctx->smem_window = max_smem_class <= (size_t)ctx->smem_optin && max_forest <= 1023 &&
                       m->cable_solver == EDEN_CABLE_BWD_EULER && !plastic_syn;

    phase("upload");
    // ---- upload
    DevModel &d = ctx->d;
    d.n_target = nt; d.n_src = m->n_src; d.n_unit = n_unit; d.n_forest = (int)fo_t0.size();
    d.n_in = (int)in_tgt.size();
    d.n_block = n_block;
    d.n_chunk = n_chunk;
    d.n_syn = ns; d.n_pois = m->n_pois; d.dt = dt;
    d.pois_exact = (dt == std::floor(dt) && dt <= 1048576.0f) ? 1 : 0;
    TRY(upload_vec(ctx, &d.v[0], v0));
    TRY(upload_vec(ctx, &d.v[1], v0));
    TRY(upload(ctx, &d.diag, (const float *)nullptr, nt));
    TRY(upload_c(ctx, &d.c_cm, c_cm)); TRY(upload_c(ctx, &d.c_inv_rc, c_inv)); TRY(upload_c(ctx, &d.c_area, c_area));
    TRY(upload_c(ctx, &d.c_u, c_u)); TRY(upload_c(ctx, &d.c_l, c_l));
    TRY(upload_c(ctx, &d.c_cend, c_cend)); TRY(upload_c(ctx, &d.c_parent, c_parent));
    d.fwd_euler = m->cable_solver == EDEN_CABLE_FWD_EULER ? 1 : 0;
    if (d.fwd_euler) {
        // each node's axial resistance to its parent and the start of its
        // child range (empty ranges start at their end)
        std::vector<float> c_rax(nt, 0.0f);
        std::vector<int32_t> c_kb(nt, 0);
        for (int it = 0; it < nt; it++) {
            const int ut = i2u[it];
            if (ut < n_comp && c_parent[it] >= 0) c_rax[it] = m->comp_r_axial[ut];
            c_kb[it] = c_nchild[it] > 0 ? c_child0[it] : c_cend[it];
        }
        TRY(upload_c(ctx, &d.c_rax, c_rax)); TRY(upload_c(ctx, &d.c_kb, c_kb));
    }
    TRY(upload_c(ctx, &d.c_kl, c_kl)); TRY(upload_c(ctx, &d.c_pv0, c_pv0));
    TRY(upload_c(ctx, &d.c_rt0, c_rt0)); TRY(upload_c(ctx, &d.c_cep, c_cep)); TRY(upload_c(ctx, &d.t_izh, t_izh));
    TRY(upload_c(ctx, &d.fo_t0, fo_t0)); TRY(upload_c(ctx, &d.fo_t1, fo_t1)); TRY(upload_c(ctx, &d.fo_l0, fo_l0));
    TRY(upload_c(ctx, &d.fo_nlev, fo_nlev)); TRY(upload_c(ctx, &d.lvl, lvl));
    {
        // double-precision forests: flags, the flat compartments' constant
        // diagonal terms, and the per-step path's double scratch
        std::vector<float> c_d0(nt, 0.0f);
        for (int it = 0; it < nt; it++)
            if (!nonflat[it]) c_d0[it] = flat_d0[it];
        TRY(upload_c(ctx, &d.fo_f64, fo_f64)); TRY(upload_c(ctx, &d.c_d0, c_d0));
        TRY(upload(ctx, &d.dscr, (const double *)nullptr, ctx->n_f64_cells > 0 ? (size_t)2 * nt : (size_t)1));
    }
    {
        // gap-junction ends per internal target, in the model's order
        std::vector<int32_t> t_gap0(nt + 1, 0), gj_peer(m->n_gap);
        std::vector<float> gj_g(m->n_gap), gj_w(m->n_gap);
        for (int64_t k = 0; k < m->n_gap; k++) t_gap0[u2i[m->gap_target[k]] + 1]++;
        for (int t = 0; t < nt; t++) t_gap0[t + 1] += t_gap0[t];
        std::vector<int32_t> fill(t_gap0.begin(), t_gap0.end() - 1);
        for (int64_t k = 0; k < m->n_gap; k++) {
            const int32_t o = fill[u2i[m->gap_target[k]]]++;
            gj_peer[o] = u2i[m->gap_peer[k]];
            gj_g[o] = m->gap_conductance[k];
            gj_w[o] = m->gap_weight[k];
        }
        TRY(upload_c(ctx, &d.t_gap0, t_gap0)); TRY(upload_c(ctx, &d.gap_peer, gj_peer));
        TRY(upload_c(ctx, &d.gap_g, gj_g)); TRY(upload_c(ctx, &d.gap_w, gj_w));
    }
    {
        // gradedSynapse ends per internal target, in the model's order; their
        // state starts at 0
        const int64_t ng = m->n_graded;
        std::vector<int32_t> t_gr0(nt + 1, 0), gr_peer(ng);
        std::vector<float> gr_par((size_t)EDEN_GRADED_PARAMS * ng), gr_w(ng), gr_s(std::max<int64_t>(ng, 1), 0.0f);
        for (int64_t k = 0; k < ng; k++) t_gr0[u2i[m->graded_target[k]] + 1]++;
        for (int t = 0; t < nt; t++) t_gr0[t + 1] += t_gr0[t];
        std::vector<int32_t> fill(t_gr0.begin(), t_gr0.end() - 1);
        for (int64_t k = 0; k < ng; k++) {
            const int32_t o = fill[u2i[m->graded_target[k]]]++;
            gr_peer[o] = u2i[m->graded_peer[k]];
            for (int j = 0; j < EDEN_GRADED_PARAMS; j++)
                gr_par[(size_t)EDEN_GRADED_PARAMS * o + j] = m->graded_params[(size_t)EDEN_GRADED_PARAMS * k + j];
            gr_w[o] = m->graded_weight[k];
        }
        TRY(upload_c(ctx, &d.t_gr0, t_gr0)); TRY(upload_c(ctx, &d.gr_peer, gr_peer));
        TRY(upload_c(ctx, &d.gr_par, gr_par)); TRY(upload_c(ctx, &d.gr_w, gr_w));
        TRY(upload_vec(ctx, &d.gr_s, gr_s));
    }
    TRY(upload_c(ctx, &d.in_tgt, in_tgt));
    TRY(upload_c(ctx, &d.t_blk0, t_blk0)); TRY(upload_c(ctx, &d.bk_kind, bk_kind));
    TRY(upload_c(ctx, &d.bk_type, bk_type)); TRY(upload_c(ctx, &d.bk_erev, bk_erev));
    TRY(upload_c(ctx, &d.bk_c0, bk_c0)); TRY(upload_c(ctx, &d.ck_blk, ck_blk));
    TRY(upload_c(ctx, &d.ck_i0, ck_i0)); TRY(upload_c(ctx, &d.ck_n, ck_n));
    TRY(upload_c(ctx, &d.ck_info, ck_info));
    TRY(upload(ctx, &d.Gp, (const float *)nullptr, (size_t)32 * (size_t)std::max(n_chunk, 1)));
    TRY(upload(ctx, &d.ck_a, (const float *)nullptr, (size_t)std::max(n_chunk, 1)));
    TRY(upload(ctx, &d.ck_b, (const float *)nullptr, (size_t)std::max(n_chunk, 1)));
    TRY(upload_c(ctx, &d.c_chan0, c_chan0)); TRY(upload_c(ctx, &d.ch_type, ch_type));
    TRY(upload_c(ctx, &d.ch_gate0, ch_gate0)); TRY(upload_c(ctx, &d.ch_gbase, ch_g)); TRY(upload_c(ctx, &d.ch_erev, ch_e));
    TRY(upload(ctx, &d.gate, (const float *)nullptr, (size_t)n_gate));
    d.n_izh = n_izh;
    TRY(upload_c(ctx, &d.iz_kind, iz_kind));
    TRY(upload_c(ctx, &d.iz_p, iz_p));
    TRY(upload(ctx, &d.iz_u, (const float *)nullptr, (size_t)n_izh));
    TRY(upload(ctx, &d.iz_s, (const float *)nullptr, (size_t)n_izh));
    TRY(upload_c(ctx, &d.pu_start, pu_s)); TRY(upload_c(ctx, &d.pu_dur, pu_d));
    TRY(upload_c(ctx, &d.pu_amp, pu_a)); TRY(upload_c(ctx, &d.pu_w, pu_w));
    TRY(upload(ctx, &d.po_ts, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_isi, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_a, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_b, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_last, (const int32_t *)nullptr, (size_t)m->n_pois));
    TRY(upload_c(ctx, &d.po_rate, po_rate)); TRY(upload_c(ctx, &d.po_w, po_w));
    TRY(upload_c(ctx, &d.po_seed, po_seed)); TRY(upload_c(ctx, &d.po_inst, po_inst));
    TRY(upload_c(ctx, &d.po_rng, po_rng));
    TRY(upload_c(ctx, &d.wv_p, wv_p));
    TRY(upload_c(ctx, &d.cl_p, cl_p));
    TRY(upload_c(ctx, &d.po_type, po_type));
    TRY(upload(ctx, &d.tm_a, (const float *)nullptr, (size_t)m->n_timed));
    TRY(upload(ctx, &d.tm_b, (const float *)nullptr, (size_t)m->n_timed));
    TRY(upload(ctx, &d.tm_last, (const int32_t *)nullptr, (size_t)m->n_timed));
    TRY(upload(ctx, &d.tm_cur, (const int64_t *)nullptr, (size_t)m->n_timed));
    TRY(upload_c(ctx, &d.tm_w, tm_w)); TRY(upload_c(ctx, &d.tm_type, tm_type));
    TRY(upload_c(ctx, &d.tm_off, tm_off)); TRY(upload_c(ctx, &d.tm_step, tm_step));
    {
        // each item's cursor starts at its first listed step
        std::vector<int64_t> cur(tm_off.begin(), tm_off.end() - 1);
        if (!cur.empty())
            CUDA_TRY(ctx, cudaMemcpy(d.tm_cur, cur.data(), sizeof(int64_t) * cur.size(), cudaMemcpyHostToDevice));
    }
    TRY(upload(ctx, &d.sy_a, (const float *)nullptr, (size_t)ns));
    {
        // blockingPlasticSynapse: plasticity state R = 1, U = p at start, and
        // each input block's voltage-block parameters
        bool any = false;
        for (int k = 0; k < m->n_syn_types; k++) any |= m->syn_types[k].kind == EDEN_SYN_BLOCKING_PLASTIC;
        std::vector<float> R(any ? ns : 1, 1.0f), U(any ? ns : 1, 1.0f);
        if (any)
            for (int64_t q = 0; q < ns; q++) U[q] = m->syn_types[sy_type[q]].release_prob;
        TRY(upload_vec(ctx, &d.sy_R, R)); TRY(upload_vec(ctx, &d.sy_U, U));
        std::vector<float2> bb(std::max<size_t>(bk_kind.size(), 1), make_float2(0.0f, 1.0f));
        for (size_t b = 0; b < bk_kind.size(); b++)
            if (bk_kind[b] & BK_BLOCK) {
                const EdenGpuSynapseType &sk = m->syn_types[bk_type[b]];
                bb[b] = make_float2(sk.block_ratio, sk.block_volt);
            }
        TRY(upload_c(ctx, &d.bk_block, bb));
    }
    TRY(upload(ctx, &d.sy_b, (const float *)nullptr, (size_t)ns));
    TRY(upload(ctx, &d.sy_last, (const int32_t *)nullptr, (size_t)ns));
    TRY(upload_vec(ctx, &d.sy_pend, sy_pend));
    TRY(upload(ctx, &d.sy_mask, (const uint32_t *)nullptr, (size_t)ns));
    TRY(upload_c(ctx, &d.sy_w, sy_w)); TRY(upload_c(ctx, &d.sy_delay, sy_d));
    TRY(upload_c(ctx, &d.sy_type, sy_type));
    ctx->h_sy_type = sy_type;
    TRY(upload_c(ctx, &d.t_src, t_src)); TRY(upload_c(ctx, &d.src_thr, src_thr));
    TRY(upload_c(ctx, &d.fan0, fan0)); TRY(upload_c(ctx, &d.fan_syn, fan_syn));
    {
        std::vector<int32_t> es(m->ext_src, m->ext_src + m->n_ext), ek((size_t)m->n_ext);
        for (int64_t k = 0; k < m->n_ext; k++) ek[(size_t)k] = (int32_t)m->ext_step[k];
        TRY(upload_c(ctx, &d.ext_src, es));
        TRY(upload_c(ctx, &d.ext_step, ek));
        ctx->h_ext_step.assign(m->ext_step, m->ext_step + m->n_ext);
    }
    // a source spikes at most once per step: a window list never exceeds n_src * K
    size_t wcap = (size_t)m->n_src * (size_t)std::max(ctx->K, 4) + 32;
    for (int b = 0; b < 2; b++) {
        TRY(upload(ctx, &d.wspk_src[b], (const int32_t *)nullptr, wcap));
        TRY(upload(ctx, &d.wspk_step[b], (const int32_t *)nullptr, wcap));
        TRY(upload(ctx, &d.wspk_time[b], (const double *)nullptr, wcap));
    }
    TRY(upload(ctx, &d.wspk_count, (const int32_t *)nullptr, 2));
    TRY(upload(ctx, &d.log_src, (const int32_t *)nullptr, (size_t)log_cap));
    TRY(upload(ctx, &d.log_step, (const int64_t *)nullptr, (size_t)log_cap));
    TRY(upload(ctx, &d.log_time, (const double *)nullptr, (size_t)log_cap));
    TRY(upload(ctx, &d.log_count, (const unsigned long long *)nullptr, 1));
    d.log_cap = log_cap;
    TRY(upload_c(ctx, &d.t_trace0, t_trace0)); TRY(upload_c(ctx, &d.trace_col, trace_col));
    TRY(upload_c(ctx, &d.trace_gate, trace_gate));
    d.n_trace = n_trace;
    TRY(upload(ctx, &d.trace_buf, (const float *)nullptr, (size_t)ctx->trace_cap * (size_t)std::max(n_trace, 1)));
    d.trace_cap = ctx->trace_cap;
    TRY(upload_c(ctx, &d.un_t0, un_t0)); TRY(upload_c(ctx, &d.un_t1, un_t1)); TRY(upload_c(ctx, &d.un_f, un_f));
    TRY(upload_c(ctx, &d.un_off, un_off)); TRY(upload_c(ctx, &d.un_gt0, un_gt0)); TRY(upload_c(ctx, &d.un_ngt, un_ngt));
    TRY(upload_c(ctx, &d.un_s0, un_s0)); TRY(upload_c(ctx, &d.un_s1, un_s1));
    TRY(upload_c(ctx, &d.un_r0, un_r0)); TRY(upload_c(ctx, &d.un_r1, un_r1)); TRY(upload_c(ctx, &d.cta_u0, cta_u0));
    TRY(upload_c(ctx, &d.gs_t, gs_t)); TRY(upload_c(ctx, &d.gs_src, gs_src)); TRY(upload_c(ctx, &d.gs_thr, gs_thr));
    TRY(upload_c(ctx, &d.gr_t, gr_t)); TRY(upload_c(ctx, &d.gr_col, gr_col));
    TRY(upload_c(ctx, &d.un_nf0, un_nf0)); TRY(upload_c(ctx, &d.un_nf1, un_nf1)); TRY(upload_c(ctx, &d.nf_t, nf_t));
    TRY(upload_c(ctx, &d.lvl_info, lvl_info)); TRY(upload_c(ctx, &d.gate_par, gate_par));
    TRY(upload_c(ctx, &d.gate_ext, gate_ext));
    TRY(upload_c(ctx, &d.nf_c0, nf_c0)); TRY(upload_c(ctx, &d.nf_c1, nf_c1)); TRY(upload_c(ctx, &d.nf_sig, nf_sig));
    TRY(upload_c(ctx, &d.nfc_g, nfc_g)); TRY(upload_c(ctx, &d.nfc_e, nfc_e));
    TRY(upload_c(ctx, &d.nfc_q, nfc_q)); TRY(upload_c(ctx, &d.nfc_i, nfc_i));
    TRY(upload(ctx, &d.status, (const int32_t *)nullptr, 1));
    TRY(upload(ctx, &ctx->d_base, (const int *)nullptr, 1));
    TRY(upload(ctx, &ctx->d_zero, (const int *)nullptr, 1));

    phase("tables");
    // ---- constant tables
    ChanTypeDev ct[kMaxChanTypes];
    memset(ct, 0, sizeof(ct));
    for (int k = 0; k < m->n_chan_types; k++) {
        const EdenGpuChannelType &s = m->chan_types[k];
        ct[k].n_gates = s.n_gates;
        for (int g = 0; g < EDEN_MAX_GATES; g++) {
            ct[k].inst[g] = s.gate_instances[g];
            ct[k].fk[g] = s.fwd_kind[g]; ct[k].fr[g] = s.fwd_rate[g]; ct[k].fm[g] = s.fwd_mid[g]; ct[k].fs[g] = s.fwd_scale[g];
            ct[k].rk[g] = s.rev_kind[g]; ct[k].rr[g] = s.rev_rate[g]; ct[k].rm[g] = s.rev_mid[g]; ct[k].rs[g] = s.rev_scale[g];
            ct[k].q10[g] = s.q10[g];
            ct[k].gk[g] = s.gate_kind[g];
            ct[k].tk[g] = s.tau_kind[g]; ct[k].tr[g] = s.tau_rate[g]; ct[k].tm[g] = s.tau_mid[g]; ct[k].ts[g] = s.tau_scale[g];
            ct[k].ik[g] = s.inf_kind[g]; ct[k].ir[g] = s.inf_rate[g]; ct[k].im[g] = s.inf_mid[g]; ct[k].is[g] = s.inf_scale[g];
        }
    }
    SynTypeDev st[kMaxSynTypes];
    memset(st, 0, sizeof(st));
    for (int k = 0; k < m->n_syn_types; k++) {
        const EdenGpuSynapseType &s = m->syn_types[k];
        st[k].kind = s.kind; st[k].gbase = s.gbase; st[k].erev = s.erev;
        st[k].tau_decay = s.tau_decay; st[k].tau_rise = s.tau_rise;
        st[k].wf_w = s.weight_prop * s.waveform_factor;
        st[k].r_decay = 1.0f / s.tau_decay;
        const bool two = s.kind == EDEN_SYN_EXPTWO || s.kind == EDEN_SYN_BLOCKING_PLASTIC;
        st[k].r_rise = two ? 1.0f / s.tau_rise : 1.0f;
        st[k].f_decay = 1.0f - dt / s.tau_decay;
        st[k].f_rise = two ? 1.0f - dt / s.tau_rise : 1.0f;
        st[k].plastic = s.kind == EDEN_SYN_BLOCKING_PLASTIC && s.tau_rec > 0.0f;
        st[k].rel_p = s.release_prob;
        st[k].f_rec = s.tau_rec > 0.0f ? 1.0f - dt / s.tau_rec : 1.0f;
        st[k].f_fac = s.tau_fac > 0.0f ? 1.0f - dt / s.tau_fac : 1.0f;
        // an alpha kind's coupling e dt / tau: g' = f g + c A per step
        st[k].c_alpha = (s.kind == EDEN_SYN_ALPHA || s.kind == EDEN_SYN_ALPHA_CURRENT)
                            ? (float)(2.7182818284590451 * (double)dt / (double)s.tau_decay) : 0.0f;
    }
    {
        const ChanTypeDev *pc = nullptr;
        const SynTypeDev *ps = nullptr;
        TRY(upload(ctx, (ChanTypeDev **)&pc, ct, kMaxChanTypes));
        TRY(upload(ctx, (SynTypeDev **)&ps, st, kMaxSynTypes));
        d.chan_types = pc;
        d.syn_types = ps;
    }
    ctx->h_syn_types.assign(st, st + kMaxSynTypes);
    // powers of each decay factor for windows without events
    {
        std::vector<float> pw((size_t)kMaxSynTypes * 2 * kPowLen, 0.0f);
        for (int k = 0; k < kMaxSynTypes; k++)
            for (int j = 0; j < kPowLen; j++) {
                pw[((size_t)k * 2 + 0) * kPowLen + j] = (float)std::pow((double)st[k].f_rise, j);
                pw[((size_t)k * 2 + 1) * kPowLen + j] = (float)std::pow((double)st[k].f_decay, j);
            }
        TRY(upload_c(ctx, &ctx->d.syn_pow, pw));
    }

    // ---- launch shapes
    auto blocks_for = [&](int64_t n) {
        int64_t b = (n + kThreads - 1) / kThreads;
        return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ctx->n_sm * 32));
    };
    ctx->grid_inputs = 1;  // set below, once the kernels are chosen
    ctx->grid_targets = blocks_for(nt);
    ctx->grid_hines = (int)std::max<int64_t>(1, ((int64_t)d.n_forest * 32 + kHinesThreads - 1) / kHinesThreads);
    ctx->grid_deliver = ctx->n_sm * 4;
    ctx->max_cell_blocks = (opt && opt->max_cell_blocks > 0) ? opt->max_cell_blocks : ctx->n_sm * 32;
    ctx->grid_window = 0;
    // per-step Hines: each warp stages a forest of up to forest_cap compartments
    // (7 arrays plus depth boundaries); larger forests are solved in place
    const int hines_warps = kHinesThreads / 32;
    ctx->forest_cap = std::min(ctx->forest_cap + 1, std::max(kForestNodes, max_forest) + 1);
    ctx->smem_hines = (size_t)hines_warps * 8 * ctx->forest_cap * sizeof(float);
    if (ctx->smem_hines > (size_t)ctx->smem_optin) {
        ctx->forest_cap = (int)(ctx->smem_optin / (hines_warps * 8 * sizeof(float)));
        ctx->smem_hines = (size_t)hines_warps * 8 * ctx->forest_cap * sizeof(float);
    }
    // windowed path: the group staging of k_cells_t; when the largest group
    // does not fit, the batched mode runs the per-step kernels instead
    // the windowed path needs every class to fit one CTA's shared memory; if
    // not, the batched mode runs the per-step kernels instead
    if (!ctx->smem_window) ctx->K = 1;
    // the windowed kernels: compiled for this model's channel sets when the
    // batched mode uses them (codegen >= 0) and NVRTC is available, else the
    // built-in ones (codegen = 1 makes a failed compile an error)
    ctx->fn_inputs = (const void *)k_inputs_t;
    ctx->fn_cells = (const void *)k_cells_t;
    ctx->fn_deliver = (const void *)k_deliver_t;
    const int codegen = opt ? opt->codegen : 0;
    if (ctx->mode == EDEN_MODE_BATCHED && ctx->smem_window && codegen >= 0) {
        phase("codegen");
        eden_codegen::Kinds kinds;
        for (int b = 0; b < n_block; b++) {
            const int kb = bk_kind[b] & BK_KIND_MASK;
            kinds.pulse |= kb == BK_PULSE && bk_type[b] == 0;
            kinds.clamp |= kb == BK_CLAMPV;
            kinds.sine |= kb == BK_PULSE && bk_type[b] == 1 + EDEN_WAVE_SINE;
            kinds.ramp |= kb == BK_PULSE && bk_type[b] == 1 + EDEN_WAVE_RAMP;
            kinds.pois |= kb == BK_POIS;
            kinds.timed |= kb == BK_TIMED;
            kinds.syn |= kb == BK_SYN;
            if (kb != BK_PULSE && kb != BK_CLAMPV) {
                const int sk = m->syn_types[bk_type[b]].kind;
                // alpha and current-based expOne items step like expOne's
                kinds.expone |= sk != EDEN_SYN_EXPTWO && sk != EDEN_SYN_BLOCKING_PLASTIC;
                kinds.exptwo |= sk == EDEN_SYN_EXPTWO || sk == EDEN_SYN_BLOCKING_PLASTIC;
                kinds.alpha |= sk == EDEN_SYN_ALPHA || sk == EDEN_SYN_ALPHA_CURRENT;
                kinds.current |= current_kind(sk);
            }
        }
        kinds.forest = d.n_forest > 0;
        kinds.gateforms = gate_forms;
        kinds.izh = n_izh > 0;
        kinds.gap = m->n_gap > 0 || m->n_graded > 0;
        ctx->codegen_source = eden_codegen::program_source(eden_codegen::kind_defines(kinds) +
                                                           eden_codegen::channel_routines(m->chan_types, chan_sets));
        eden_codegen::Kernels kk;
        std::string why;
        if (eden_codegen::compile(ctx->codegen_source, ctx->device, kk, why, ctx->codegen_ms)) {
            ctx->fn_inputs = kk.inputs;
            ctx->fn_cells = kk.cells;
            ctx->fn_deliver = kk.deliver;
            ctx->codegen_used = true;
        } else {
            ctx->codegen_note = why;
            if (codegen == 1) return ctx->fail(EDEN_GPU_E_CUDA, "code generation failed: %s", why.c_str());
        }
    }
    CUDA_TRY(ctx, cudaFuncSetAttribute(k_hines_t, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_hines));
    if (ctx->smem_window)
        CUDA_TRY(ctx, cudaFuncSetAttribute(ctx->fn_cells, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)std::min<size_t>(max_smem_class, (size_t)ctx->smem_optin)));
    {
        // resident input blocks only: each warp then walks several chunks
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ctx->fn_inputs, kInputThreads, 0);
        ctx->grid_inputs = (int)std::max<int64_t>(
            1, std::min<int64_t>(((int64_t)ctx->d.n_chunk * 32 + kInputThreads - 1) / kInputThreads,
                                 (int64_t)ctx->n_sm * std::max(per_sm, 1)));
    }
    phase("done");
    if (verbose) {
        fprintf(stderr, "libeden_gpu: set-up %s\n", timing.c_str());
        int occ_cells = 0, occ_inputs = 0;
        if (ctx->smem_window)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_cells, ctx->fn_cells, kCellThreads, max_smem_class);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_inputs, ctx->fn_inputs, kInputThreads, 0);
        fprintf(stderr, "libeden_gpu: kernels %s%s%s (%.0f ms)\n",
                ctx->codegen_used ? "compiled for this model" : "built in",
                ctx->codegen_note.empty() ? "" : ": ", ctx->codegen_note.c_str(), ctx->codegen_ms);
        int64_t fnodes = 0, flev = 0;
        for (size_t f = 0; f < fo_t0.size(); f++) { fnodes += fo_t1[f] - fo_t0[f]; flev += fo_nlev[f]; }
        fprintf(stderr,
                "libeden_gpu: %d targets, %d cells, %lld synapses, %lld poisson, %d blocks, %d input targets\n"
                "libeden_gpu: K=%d, %d CTAs (%d thr, up to %zu B smem, %d/SM at the largest), %zu forests "
                "(%.1f nodes, %.1f levels avg)\n"
                "libeden_gpu: %d units, %zu size classes; inputs grid %d (%d/SM)\n",
                nt, m->n_src, (long long)ns, (long long)m->n_pois, n_block, (int)in_tgt.size(), ctx->K,
                (int)cta_words.size(), kCellThreads, max_smem_class, occ_cells, fo_t0.size(),
                fo_t0.empty() ? 0.0 : (double)fnodes / fo_t0.size(), fo_t0.empty() ? 0.0 : (double)flev / fo_t0.size(),
                n_unit, ctx->classes.size(), ctx->grid_inputs, occ_inputs);
    }
    return 0;
}

extern "C" int edenGpuCreate(const EdenGpuModel *model, const EdenGpuOptions *opt, EdenGpuCtx **out) {
    if (!out) return EDEN_GPU_E_INVALID;
    *out = nullptr;
    EdenGpuCtx *ctx = new EdenGpuCtx();
    *out = ctx;
    if (!model) return ctx->fail(EDEN_GPU_E_INVALID, "null model");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return ctx->fail(EDEN_GPU_E_NODEVICE, "no CUDA device visible");
    }
    ctx->device = opt ? opt->device : 0;
    if (ctx->device < 0 || ctx->device >= ndev) return ctx->fail(EDEN_GPU_E_INVALID, "device %d not present", ctx->device);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    TRY(validate(ctx, model));
    if (opt && opt->n_trace > 0 && !opt->trace_target) return ctx->fail(EDEN_GPU_E_INVALID, "trace_target missing");
    CUDA_TRY(ctx, cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
    CUDA_TRY(ctx, cudaDeviceGetAttribute(&ctx->smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
    CUDA_TRY(ctx, cudaDeviceGetAttribute(&ctx->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CUDA_TRY(ctx, cudaEventCreate(&ctx->ev0));
    CUDA_TRY(ctx, cudaEventCreate(&ctx->ev1));
    TRY(build_and_upload(ctx, model, opt));
    CUDA_TRY(ctx, cudaDeviceSynchronize());
    return 0;
}

// ---------------------------------------------------------------------------
static int ensure_wtab(EdenGpuCtx *ctx, int64_t n) {
    if (n <= ctx->wtab_cap) return 0;
    int64_t cap = std::max<int64_t>(n, 1024);
    // the captured graph refers to the old tables: capture it again
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    if (ctx->h_wtab) cudaFreeHost(ctx->h_wtab);
    if (ctx->h_wtimes) cudaFreeHost(ctx->h_wtimes);
    ctx->h_wtab = nullptr;
    ctx->h_wtimes = nullptr;
    for (void *old : {(void *)ctx->d_wtab, (void *)ctx->d_wtimes}) {
        if (!old) continue;
        cudaFree(old);
        ctx->allocs.erase(std::remove(ctx->allocs.begin(), ctx->allocs.end(), old), ctx->allocs.end());
    }
    CUDA_TRY(ctx, cudaMallocHost(&ctx->h_wtab, sizeof(WindowArgs) * cap));
    CUDA_TRY(ctx, cudaMallocHost(&ctx->h_wtimes, sizeof(WindowTimes) * cap));
    void *p = nullptr, *q = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&p, sizeof(WindowArgs) * cap));
    ctx->allocs.push_back(p);
    CUDA_TRY(ctx, cudaMalloc(&q, sizeof(WindowTimes) * cap));
    ctx->allocs.push_back(q);
    ctx->d_wtab = (WindowArgs *)p;
    ctx->d_wtimes = (WindowTimes *)q;
    ctx->wtab_cap = cap;
    return 0;
}

// The next window's arguments and step times (in double from the host
// clock, as the reference accumulates time, eden/Eden.cpp:11486, 11931), and
// the host clock advanced past it; the previous window's times are kept for
// the trigger replay.
static void fill_window(EdenGpuCtx *ctx, WindowArgs &w, WindowTimes &tt, int64_t s, int K) {
    w.t0 = ctx->time;
    w.step0 = s;
    w.K = K;
    w.Kprev = ctx->Kprev;
    w.par = ctx->par;
    w.wpar = ctx->wpar;
    {
        const auto &es = ctx->h_ext_step;
        w.ext0 = (int32_t)(std::lower_bound(es.begin(), es.end(), s + 1) - es.begin());
        w.ext1 = (int32_t)(std::lower_bound(es.begin(), es.end(), s + K + 1) - es.begin());
    }
    double t = ctx->time;
    for (int j = 0; j < 32; j++) {
        tt.tk[j] = (float)t;
        tt.tprev[j] = ctx->prev_tk[j];
        if (s + j > 0) t += (double)ctx->d.dt;
    }
    if (s > 0) {
        ctx->t_prev0 = ctx->time;
        ctx->Kprev = K;
        for (int k = 0; k < K; k++) ctx->time += (double)ctx->d.dt;
        for (int j = 0; j < 32; j++) ctx->prev_tk[j] = tt.tk[j];
    }
    ctx->par ^= (K & 1);
    ctx->wpar ^= 1;
}

// The host clock and buffer parities fill_window advances, saved at the
// start of a run so that a run that fails before any kernel is issued leaves
// the context as it was.
struct ClockState {
    double time, t_prev0;
    int par, wpar, Kprev;
    float prev_tk[32];
};
static ClockState save_clock(const EdenGpuCtx *ctx) {
    ClockState c{ctx->time, ctx->t_prev0, ctx->par, ctx->wpar, ctx->Kprev, {}};
    std::copy(ctx->prev_tk, ctx->prev_tk + 32, c.prev_tk);
    return c;
}
static void restore_clock(EdenGpuCtx *ctx, const ClockState &c) {
    ctx->time = c.time;
    ctx->t_prev0 = c.t_prev0;
    ctx->par = c.par;
    ctx->wpar = c.wpar;
    ctx->Kprev = c.Kprev;
    std::copy(c.prev_tk, c.prev_tk + 32, ctx->prev_tk);
}

// A run's outcome: on failure before any kernel was issued the clock is put
// back (the same first_step can be retried); on failure after, with the
// steps not completed, the context refuses later runs.
static int finish_run(EdenGpuCtx *ctx, int rc, const ClockState &c, int64_t next_before) {
    if (rc != 0 && ctx->next_step == next_before) {
        if (!ctx->launched) restore_clock(ctx, c);
        else ctx->broken = true;
    }
    return rc;
}

static int check_runnable(EdenGpuCtx *ctx) {
    if (ctx->broken)
        return ctx->fail(EDEN_GPU_E_CUDA, "an earlier run failed after launching its kernels (%s); the device state "
                                          "is not the host's, destroy the context",
                         ctx->err.c_str());
    ctx->launched = false;
    return 0;
}

// Event pair around a launch when kernel timing is on.
static void tmark(EdenGpuCtx *ctx, int kind, bool before) {
    if (!ctx->kernel_timing) return;
    if (before) {
        if (ctx->tev_used + 2 > ctx->tev.size()) {
            for (int k = 0; k < 64; k++) {
                cudaEvent_t e;
                cudaEventCreate(&e);
                ctx->tev.push_back(e);
                ctx->tev_kind.push_back(0);
            }
        }
        ctx->tev_kind[ctx->tev_used] = kind;
        cudaEventRecord(ctx->tev[ctx->tev_used], ctx->stream);
    } else {
        cudaEventRecord(ctx->tev[ctx->tev_used + 1], ctx->stream);
        ctx->tev_used += 2;
    }
}

// Launch the kernels of window `idx` of the current table; returns launches.
static int launch_window(EdenGpuCtx *ctx, const int *base, int idx, int K) {
    ctx->launched = true;
    DevModel &d = ctx->d;
    cudaStream_t s = ctx->stream;
    if (ctx->mode == EDEN_MODE_BATCHED && ctx->smem_window) {
        tmark(ctx, EDEN_KERNEL_INPUTS, true);
        launch_k(ctx->fn_inputs, ctx->grid_inputs, kInputThreads, 0, s, d, (const WindowArgs *)ctx->d_wtab,
                 (const WindowTimes *)ctx->d_wtimes, base, idx);
        tmark(ctx, EDEN_KERNEL_INPUTS, false);
        int n = 1;
        tmark(ctx, EDEN_KERNEL_CELLS, true);
        for (const auto &cl : ctx->classes) {
            const int nb = std::min(cl.cta_end - cl.cta_begin, ctx->max_cell_blocks);
            launch_k(ctx->fn_cells, nb, kCellThreads, cl.smem, s, d, (const WindowArgs *)ctx->d_wtab,
                     (const WindowTimes *)ctx->d_wtimes, base, idx, cl.cta_begin, cl.cta_end);
            n++;
        }
        tmark(ctx, EDEN_KERNEL_CELLS, false);
        tmark(ctx, EDEN_KERNEL_DELIVER, true);
        launch_k(ctx->fn_deliver, ctx->grid_deliver, kThreads, 0, s, d, (const WindowArgs *)ctx->d_wtab, base, idx);
        tmark(ctx, EDEN_KERNEL_DELIVER, false);
        return n + 1;
    }
    (void)K;
    tmark(ctx, EDEN_KERNEL_INPUTS, true);
    launch_k(ctx->fn_inputs, ctx->grid_inputs, kInputThreads, 0, s, d, (const WindowArgs *)ctx->d_wtab,
             (const WindowTimes *)ctx->d_wtimes, base, idx);
    tmark(ctx, EDEN_KERNEL_INPUTS, false);
    tmark(ctx, EDEN_KERNEL_TARGETS, true);
    k_targets_t<<<ctx->grid_targets, kThreads, 0, s>>>(d, ctx->d_wtab, ctx->d_wtimes, base, idx);
    tmark(ctx, EDEN_KERNEL_TARGETS, false);
    tmark(ctx, EDEN_KERNEL_HINES, true);
    k_hines_t<<<ctx->grid_hines, kHinesThreads, ctx->smem_hines, s>>>(d, ctx->d_wtab, base, idx, ctx->forest_cap);
    tmark(ctx, EDEN_KERNEL_HINES, false);
    tmark(ctx, EDEN_KERNEL_DELIVER, true);
    launch_k(ctx->fn_deliver, ctx->grid_deliver, kThreads, 0, s, d, (const WindowArgs *)ctx->d_wtab, base, idx);
    tmark(ctx, EDEN_KERNEL_DELIVER, false);
    return 4;
}

static int run_windows(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps);

extern "C" int edenGpuRun(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    TRY(check_runnable(ctx));
    const ClockState c = save_clock(ctx);
    const int64_t next_before = ctx->next_step;
    return finish_run(ctx, run_windows(ctx, first_step, n_steps), c, next_before);
}

static int run_windows(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps) {
    if (n_steps < 0) return ctx->fail(EDEN_GPU_E_INVALID, "negative step count");
    if (first_step != ctx->next_step)
        return ctx->fail(EDEN_GPU_E_INVALID, "steps must be contiguous: expected first_step %lld",
                         (long long)ctx->next_step);
    int64_t last = first_step + n_steps - 1;
    int64_t rec_first = std::max<int64_t>(first_step, 1);
    if (last >= rec_first && last - ctx->trace_first_unfetched + 1 > ctx->trace_cap)
        return ctx->fail(EDEN_GPU_E_RANGE, "trajectory buffer holds %lld steps; fetch records first",
                         (long long)ctx->trace_cap);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // window schedule: the 4 initialisation passes, then windows of K
    std::vector<Window> wins;
    int64_t s = first_step;
    while (s <= last) {
        int K;
        if (ctx->mode != EDEN_MODE_BATCHED) K = 1;
        else if (s <= 0) K = (int)std::min<int64_t>(-s + 1, last - s + 1);
        else K = (int)std::min<int64_t>(ctx->K, last - s + 1);
        wins.push_back({s, K});
        s += K;
    }
    TRY(ensure_wtab(ctx, (int64_t)wins.size() + kGraphWindows));
    for (size_t i = 0; i < wins.size(); i++) fill_window(ctx, ctx->h_wtab[i], ctx->h_wtimes[i], wins[i].step0, wins[i].K);
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_wtab, ctx->h_wtab, sizeof(WindowArgs) * wins.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_wtimes, ctx->h_wtimes, sizeof(WindowTimes) * wins.size(),
                                  cudaMemcpyHostToDevice, ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_base, 0, sizeof(int), ctx->stream));
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    int64_t launches = 0;
    size_t i = 0;
    ctx->tev_used = 0;
    // graph replay for full chunks of regular windows (batched mode)
    if (ctx->mode == EDEN_MODE_BATCHED && !ctx->kernel_timing) {
        while (i < wins.size() && wins[i].step0 <= 0) {
            launches += launch_window(ctx, ctx->d_zero, (int)i, wins[i].K);
            i++;
        }
        // align the device chunk base with the first regular window
        if (i > 0) {
            k_bump<<<1, 1, 0, ctx->stream>>>(ctx->d_base, (int)i);
            launches++;
        }
        while (i + kGraphWindows <= wins.size()) {
            bool uniform = true;
            for (int j = 0; j < kGraphWindows; j++) uniform &= wins[i + j].K == ctx->K;
            if (!uniform) break;
            if (!ctx->graph) {
                cudaGraph_t g;
                CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
                for (int j = 0; j < kGraphWindows; j++) launch_window(ctx, ctx->d_base, j, ctx->K);
                k_bump<<<1, 1, 0, ctx->stream>>>(ctx->d_base, kGraphWindows);
                CUDA_TRY(ctx, cudaStreamEndCapture(ctx->stream, &g));
                CUDA_TRY(ctx, cudaGraphInstantiate(&ctx->graph, g, 0));
                cudaGraphDestroy(g);
            }
            ctx->launched = true;
            CUDA_TRY(ctx, cudaGraphLaunch(ctx->graph, ctx->stream));
            launches += kGraphWindows * (2 + (int64_t)ctx->classes.size()) + 1;
            i += kGraphWindows;
        }
    }
    for (; i < wins.size(); i++) launches += launch_window(ctx, ctx->d_zero, (int)i, wins[i].K);
    CUDA_TRY(ctx, cudaGetLastError());
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->last_launches = launches;
    for (size_t e = 0; e < ctx->tev_used; e += 2) {
        float kms = 0;
        CUDA_TRY(ctx, cudaEventElapsedTime(&kms, ctx->tev[e], ctx->tev[e + 1]));
        ctx->k_ms[ctx->tev_kind[e]] += kms;
        ctx->k_n[ctx->tev_kind[e]]++;
    }
    ctx->next_step = last + 1;
    int status = 0;
    CUDA_TRY(ctx, cudaMemcpy(&status, ctx->d.status, sizeof(int), cudaMemcpyDeviceToHost));
    ctx->sticky_status |= status;
    if (status & ST_LOG_OVERFLOW) return ctx->fail(EDEN_GPU_E_RANGE, "spike log overflow; fetch records more often");
    return 0;
}

extern "C" int edenGpuKernelStats(EdenGpuCtx *ctx, int32_t kind, double *total_ms, int64_t *launches) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    if (kind < 0 || kind >= EDEN_KERNEL_KINDS) return ctx->fail(EDEN_GPU_E_RANGE, "kernel kind %d", kind);
    if (total_ms) *total_ms = ctx->k_ms[kind];
    if (launches) *launches = ctx->k_n[kind];
    return 0;
}

extern "C" int edenGpuFp64Cells(EdenGpuCtx *ctx, int64_t *n_cells) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    if (n_cells) *n_cells = ctx->n_f64_cells;
    return 0;
}

extern "C" int edenGpuLastRunStats(EdenGpuCtx *ctx, double *device_ms, int64_t *launches) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    if (device_ms) *device_ms = ctx->last_ms;
    if (launches) *launches = ctx->last_launches;
    return 0;
}

extern "C" int edenGpuFetchRecords(EdenGpuCtx *ctx, EdenGpuRecords *rec) {
    if (!ctx || !rec) return EDEN_GPU_E_INVALID;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    int64_t first = ctx->trace_first_unfetched;
    int64_t last = ctx->next_step - 1;  // last completed step
    int64_t n = std::max<int64_t>(0, last - first + 1);
    if (n > rec->trace_capacity) return ctx->fail(EDEN_GPU_E_RANGE, "trace buffer too small (%lld rows needed)", (long long)n);
    int nt = ctx->n_trace;
    std::vector<float> host((size_t)ctx->trace_cap * std::max(nt, 1));
    if (n > 0 && nt > 0) {
        CUDA_TRY(ctx, cudaMemcpy(host.data(), ctx->d.trace_buf, sizeof(float) * host.size(), cudaMemcpyDeviceToHost));
        for (int64_t k = 0; k < n; k++) {
            int64_t step = first + k;
            int64_t row = (step - 1) % ctx->trace_cap;
            memcpy(rec->trace + k * nt, host.data() + row * nt, sizeof(float) * nt);
            if (rec->trace_step) rec->trace_step[k] = step;
        }
    } else if (rec->trace_step) {
        for (int64_t k = 0; k < n; k++) rec->trace_step[k] = first + k;
    }
    rec->n_trace_samples = n;
    ctx->trace_first_unfetched = last + 1;
    unsigned long long cnt = 0;
    CUDA_TRY(ctx, cudaMemcpy(&cnt, ctx->d.log_count, sizeof(cnt), cudaMemcpyDeviceToHost));
    int64_t ns = (int64_t)std::min<unsigned long long>(cnt, (unsigned long long)ctx->d.log_cap);
    if (ns > rec->spike_capacity) return ctx->fail(EDEN_GPU_E_RANGE, "spike buffer too small (%lld needed)", (long long)ns);
    if (ns > 0) {
        CUDA_TRY(ctx, cudaMemcpy(rec->spike_src, ctx->d.log_src, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost));
        CUDA_TRY(ctx, cudaMemcpy(rec->spike_step, ctx->d.log_step, sizeof(int64_t) * ns, cudaMemcpyDeviceToHost));
        if (rec->spike_time_us)
            CUDA_TRY(ctx, cudaMemcpy(rec->spike_time_us, ctx->d.log_time, sizeof(double) * ns, cudaMemcpyDeviceToHost));
    }
    rec->n_spikes = ns;
    CUDA_TRY(ctx, cudaMemset(ctx->d.log_count, 0, sizeof(unsigned long long)));
    int status = ctx->sticky_status;
    ctx->sticky_status = 0;
    CUDA_TRY(ctx, cudaMemset(ctx->d.status, 0, sizeof(int)));
    if (status & ST_LOG_OVERFLOW) return ctx->fail(EDEN_GPU_E_RANGE, "spike log overflowed since the last fetch");
    if (n > 0 && nt > 0)
        for (int64_t k = 0; k < n * nt; k++)
            if (!std::isfinite(rec->trace[k])) return ctx->fail(EDEN_GPU_E_NONFINITE, "non-finite recorded value");
    return 0;
}

extern "C" int edenGpuReadV(EdenGpuCtx *ctx, float *v_host, int64_t n) {
    if (!ctx || !v_host) return EDEN_GPU_E_INVALID;
    if (n != ctx->n_target) return ctx->fail(EDEN_GPU_E_RANGE, "expected %d values", ctx->n_target);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<float> tmp(n);
    CUDA_TRY(ctx, cudaMemcpy(tmp.data(), ctx->d.v[ctx->par], sizeof(float) * n, cudaMemcpyDeviceToHost));
    for (int64_t u = 0; u < n; u++) v_host[u] = tmp[ctx->user_to_internal[u]];
    return 0;
}

extern "C" int edenGpuWriteV(EdenGpuCtx *ctx, const float *v_host, int64_t n) {
    if (!ctx || !v_host) return EDEN_GPU_E_INVALID;
    if (n != ctx->n_target) return ctx->fail(EDEN_GPU_E_RANGE, "expected %d values", ctx->n_target);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<float> tmp(n);
    for (int64_t u = 0; u < n; u++) tmp[ctx->user_to_internal[u]] = v_host[u];
    CUDA_TRY(ctx, cudaMemcpy(ctx->d.v[ctx->par], tmp.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    return 0;
}

extern "C" int edenGpuReadSynapses(EdenGpuCtx *ctx, float *pending_us, float *state_a, float *state_b, int64_t n) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    if (n != ctx->n_syn) return ctx->fail(EDEN_GPU_E_RANGE, "expected %lld synapses", (long long)ctx->n_syn);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (n == 0) return 0;
    std::vector<float> pend(n), a(n), b(n);
    std::vector<int32_t> last(n);
    CUDA_TRY(ctx, cudaMemcpy(pend.data(), ctx->d.sy_pend, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CUDA_TRY(ctx, cudaMemcpy(a.data(), ctx->d.sy_a, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CUDA_TRY(ctx, cudaMemcpy(b.data(), ctx->d.sy_b, sizeof(float) * n, cudaMemcpyDeviceToHost));
    CUDA_TRY(ctx, cudaMemcpy(last.data(), ctx->d.sy_last, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    // each synapse keeps its state as of its last event; decay it to the
    // start of the next step the way the kernel does for its next event
    for (int64_t u = 0; u < n; u++) {
        const int64_t k = ctx->syn_internal_of_user[u];
        const SynTypeDev &st = ctx->h_syn_types[ctx->h_sy_type[k]];
        const int64_t steps = std::max<int64_t>(0, ctx->next_step - (int64_t)last[k] - 1);
        const bool two = st.kind == EDEN_SYN_EXPTWO || st.kind == EDEN_SYN_BLOCKING_PLASTIC;
        if (pending_us) pending_us[u] = pend[k];
        if (state_a) state_a[u] = steps > 0 ? a[k] * powf(two ? st.f_rise : st.f_decay, (float)steps) : a[k];
        if (state_b) state_b[u] = two ? (steps > 0 ? b[k] * powf(st.f_decay, (float)steps) : b[k]) : 0.0f;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// edenGpuRunStaticScratch: edenGpuRun without any allocation.
//
// edenGpuRun can allocate while it runs: it grows the window table (device
// memory and pinned host memory) when one call spans more windows than the
// table holds, and the first batched call instantiates a CUDA graph.  A
// caller that has handed the simulator a fixed device-memory budget up front
// (a co-simulation beside other GPU code that owns the rest of HBM), or a
// host loop that must not stall on cudaMalloc/cudaFree (both can synchronise
// the whole device), cannot accept that.  This entry point runs the same
// kernels in the same order as edenGpuRun, with
//   - the input kernel's per-window conductance scratch (32 rows of n_chunk
//     floats) in the file-scope array g_static_gp instead of the context's
//     buffer, which limits it to models of at most kStaticGpChunks input
//     chunks (16 MiB of scratch); larger models get EDEN_GPU_E_RANGE;
//   - the window arguments and step times in the file-scope tables
//     g_static_wtab and g_static_wtimes, filled from stack buffers at most
//     kStaticWindows windows at a time;
//   - plain launches: no graph, no kernel-timing events.
// The first call on a context looks up the arrays' device addresses with
// cudaGetSymbolAddress, with the context's device current.  That set-up
// should happen before any stream capture begins: a call with n_steps = 0
// does only it.  The arrays belong to the library's module: every device
// that loads it holds them (16 MiB and a few KB) until the process exits,
// whether or not this entry point is ever called.
// Nothing in either array has to start at zero: every window writes rows
// 0..K-1 of every chunk before the cell kernels read them, and each launch
// reads only table entries written by the copy before it.
// The arrays exist once per device, not per context: calls that overlap in
// time on one device (two threads, or two contexts on different streams)
// race on them, so the caller must serialise such calls.
// ---------------------------------------------------------------------------
namespace {
constexpr int kStaticGpChunks = 131072;  // input chunks the static scratch holds
constexpr int kStaticWindows = 64;       // window arguments copied per batch
}  // namespace

static __device__ __align__(256) float g_static_gp[32 * kStaticGpChunks];
static __device__ __align__(256) WindowArgs g_static_wtab[kStaticWindows];
static __device__ __align__(256) WindowTimes g_static_wtimes[kStaticWindows];

// Device addresses of the static arrays on ctx's device (which is current),
// looked up on the context's first call.  A context does not outlive its
// device's primary context (a device reset frees its buffers), so the
// addresses it keeps stay valid for as long as it can run.
static int static_scratch(EdenGpuCtx *ctx, float **gp, WindowArgs **tab, WindowTimes **times) {
    if (!ctx->static_gp) {
        void *p = nullptr, *q = nullptr, *r = nullptr;
        CUDA_TRY(ctx, cudaGetSymbolAddress(&p, g_static_gp));
        CUDA_TRY(ctx, cudaGetSymbolAddress(&q, g_static_wtab));
        CUDA_TRY(ctx, cudaGetSymbolAddress(&r, g_static_wtimes));
        ctx->static_gp = (float *)p;
        ctx->static_tab = (WindowArgs *)q;
        ctx->static_times = (WindowTimes *)r;
    }
    *gp = ctx->static_gp;
    *tab = ctx->static_tab;
    *times = ctx->static_times;
    return 0;
}

// The launches of launch_window for window `idx` of `tab`, with the model
// `dm` (the context's, scratch pointer replaced) and without timing marks.
static int launch_window_static(EdenGpuCtx *ctx, const DevModel &dm, const WindowArgs *tab, const WindowTimes *times,
                                int idx) {
    ctx->launched = true;
    cudaStream_t s = ctx->stream;
    const int *zero = ctx->d_zero;
    if (ctx->mode == EDEN_MODE_BATCHED && ctx->smem_window) {
        launch_k(ctx->fn_inputs, ctx->grid_inputs, kInputThreads, 0, s, dm, tab, times, zero, idx);
        int n = 1;
        for (const auto &cl : ctx->classes) {
            const int nb = std::min(cl.cta_end - cl.cta_begin, ctx->max_cell_blocks);
            launch_k(ctx->fn_cells, nb, kCellThreads, cl.smem, s, dm, tab, times, zero, idx, cl.cta_begin,
                     cl.cta_end);
            n++;
        }
        launch_k(ctx->fn_deliver, ctx->grid_deliver, kThreads, 0, s, dm, tab, zero, idx);
        return n + 1;
    }
    launch_k(ctx->fn_inputs, ctx->grid_inputs, kInputThreads, 0, s, dm, tab, times, zero, idx);
    k_targets_t<<<ctx->grid_targets, kThreads, 0, s>>>(dm, tab, times, zero, idx);
    k_hines_t<<<ctx->grid_hines, kHinesThreads, ctx->smem_hines, s>>>(dm, tab, zero, idx, ctx->forest_cap);
    launch_k(ctx->fn_deliver, ctx->grid_deliver, kThreads, 0, s, dm, tab, zero, idx);
    return 4;
}

static int run_static(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps);

extern "C" int edenGpuRunStaticScratch(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps) {
    if (!ctx) return EDEN_GPU_E_INVALID;
    TRY(check_runnable(ctx));
    const ClockState c = save_clock(ctx);
    const int64_t next_before = ctx->next_step;
    return finish_run(ctx, run_static(ctx, first_step, n_steps), c, next_before);
}

static int run_static(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps) {
    if (n_steps < 0) return ctx->fail(EDEN_GPU_E_INVALID, "negative step count");
    if (first_step != ctx->next_step)
        return ctx->fail(EDEN_GPU_E_INVALID, "steps must be contiguous: expected first_step %lld",
                         (long long)ctx->next_step);
    if (ctx->d.n_chunk > kStaticGpChunks)
        return ctx->fail(EDEN_GPU_E_RANGE,
                         "edenGpuRunStaticScratch: the model has %d input chunks but the static scratch holds %d "
                         "(%d MiB); run it with edenGpuRun",
                         ctx->d.n_chunk, kStaticGpChunks, (int)(sizeof(float) * 32 * kStaticGpChunks >> 20));
    const int64_t last = first_step + n_steps - 1;
    const int64_t rec_first = std::max<int64_t>(first_step, 1);
    if (last >= rec_first && last - ctx->trace_first_unfetched + 1 > ctx->trace_cap)
        return ctx->fail(EDEN_GPU_E_RANGE, "trajectory buffer holds %lld steps; fetch records first",
                         (long long)ctx->trace_cap);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    float *gp = nullptr;
    WindowArgs *tab = nullptr;
    WindowTimes *times = nullptr;
    TRY(static_scratch(ctx, &gp, &tab, &times));
    if (n_steps == 0) return 0;
    DevModel dm = ctx->d;
    dm.Gp = gp;
    WindowArgs batch[kStaticWindows];
    WindowTimes tbatch[kStaticWindows];
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    int64_t launches = 0;
    int64_t s = first_step;
    while (s <= last) {
        // the same window schedule and bookkeeping as edenGpuRun
        int nb = 0;
        while (nb < kStaticWindows && s <= last) {
            int K;
            if (ctx->mode != EDEN_MODE_BATCHED) K = 1;
            else if (s <= 0) K = (int)std::min<int64_t>(-s + 1, last - s + 1);
            else K = (int)std::min<int64_t>(ctx->K, last - s + 1);
            fill_window(ctx, batch[nb], tbatch[nb], s, K);
            nb++;
            s += K;
        }
        // stream-ordered after the previous batch's launches, so the table is
        // not overwritten while they read it; the stack buffer is free for
        // reuse once the copy call returns
        CUDA_TRY(ctx, cudaMemcpyAsync(tab, batch, sizeof(WindowArgs) * nb, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_TRY(ctx, cudaMemcpyAsync(times, tbatch, sizeof(WindowTimes) * nb, cudaMemcpyHostToDevice, ctx->stream));
        for (int i = 0; i < nb; i++) launches += launch_window_static(ctx, dm, tab, times, i);
        CUDA_TRY(ctx, cudaGetLastError());
    }
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->last_ms = ms;
    ctx->last_launches = launches;
    ctx->next_step = last + 1;
    int status = 0;
    CUDA_TRY(ctx, cudaMemcpy(&status, ctx->d.status, sizeof(int), cudaMemcpyDeviceToHost));
    ctx->sticky_status |= status;
    if (status & ST_LOG_OVERFLOW) return ctx->fail(EDEN_GPU_E_RANGE, "spike log overflow; fetch records more often");
    return 0;
}
