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
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/eden_gpu.h"
#include "eden_kernels.cuh"

using namespace eden;

namespace {

constexpr int kThreads = 256;
constexpr int kGraphWindows = 16;  // windows per captured graph

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
    int64_t wtab_cap = 0;
    int *d_base = nullptr;      // chunk base read by graph-launched kernels
    int *d_zero = nullptr;      // always 0, for direct launches
    cudaGraphExec_t graph = nullptr;
    int grid_inputs = 0, grid_targets = 0, grid_hines = 0, grid_deliver = 0, grid_window = 0;
    int n_sm_unused = 0;
    int smem_per_sm = 0, smem_optin = 0;   // bytes
    int gcap = 0, forest_cap = 0;          // targets per group / compartments per forest
    bool smem_window = false;              // groups fit shared memory
    size_t smem_hines = 0, smem_win = 0;
    double last_ms = 0.0;
    int64_t last_launches = 0;
    int sticky_status = 0;

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

// ---------------------------------------------------------------------------
// kernels; each reads its WindowArgs from a device table so that a captured
// graph can be replayed over many windows
// ---------------------------------------------------------------------------
namespace eden {

// Per-step path, phase 1: one warp per target with inputs.
__global__ void __launch_bounds__(256) k_inputs_t(DevModel m, const WindowArgs *tab, const int *base, int idx) {
    const WindowArgs w = tab[*base + idx];
    const float *vin = m.v[w.par];
    const float t = (float)w.t0;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int ii = warp; ii < m.n_in; ii += nwarps) {
        int tg = m.in_tgt[ii];
        float Iin, Gin, Isyn, Gsyn;
        inputs_warp(m, tg, w, w.step0, t, true, vin[tg], Iin, Gin, Isyn, Gsyn);
        if ((threadIdx.x & 31) == 0) {
            m.in_I[tg] = Iin; m.in_G[tg] = Gin; m.syn_I[tg] = Isyn; m.syn_G[tg] = Gsyn;
        }
    }
}

// Per-step path, phase 2: one thread per target.
__global__ void __launch_bounds__(256) k_targets_t(DevModel m, const WindowArgs *tab, const int *base, int idx) {
    const WindowArgs w = tab[*base + idx];
    const bool init = w.step0 <= 0;
    const float *vin = m.v[w.par];
    float *vout = m.v[w.par ^ 1];
    const int n = m.n_target;
    const int nround = (n + 31) & ~31;  // whole warps stay converged for the spike ballot
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += gridDim.x * blockDim.x)
        if (i < n) target_step(m, i, init, w.step0, vin[i], m.in_I[i], m.in_G[i], m.syn_I[i], m.syn_G[i],
                               &vout[i], &m.diag[i], w.wpar);
}

// Per-step path, phase 3: one warp per forest, staged in shared memory when
// the forest fits its warp's slice (cap floats per array), else in place.
__global__ void __launch_bounds__(256) k_hines_t(DevModel m, const WindowArgs *tab, const int *base, int idx, int cap) {
    extern __shared__ float sm[];
    const WindowArgs w = tab[*base + idx];
    const bool init = w.step0 <= 0;
    const float *vin = m.v[w.par];
    float *x = m.v[w.par ^ 1];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    float *sD = sm + (size_t)wib * 5 * cap, *sX = sD + cap, *sU = sX + cap, *sL = sU + cap, *sV = sL + cap;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int f = warp; f < m.n_forest; f += nwarps) {
        const int c0 = m.fo_t0[f], n = m.fo_t1[f] - c0;
        if (n <= cap) {
            for (int i = lane; i < n; i += 32) {
                sD[i] = m.diag[c0 + i]; sX[i] = x[c0 + i]; sU[i] = m.c_u[c0 + i];
                sL[i] = m.c_l[c0 + i]; sV[i] = vin[c0 + i];
            }
            __syncwarp();
            hines_forest(m, f, init, w.step0, sD, sX, sU, sL, sV, c0, w.wpar);
            __syncwarp();
            for (int i = lane; i < n; i += 32) x[c0 + i] = sX[i];
            __syncwarp();
        } else {
            hines_forest(m, f, init, w.step0, m.diag, x, m.c_u, m.c_l, vin, 0, w.wpar);
        }
    }
}

// Fan the spikes of window `w` out to their synapses' trigger masks
// (bit = logging step - window start = the step at which the reference reads
// the trigger, eden/Eden.cpp:3964-3992) and append them to the spike log.
__global__ void __launch_bounds__(256) k_deliver_t(DevModel m, const WindowArgs *tab, const int *base, int idx) {
    const WindowArgs w = tab[*base + idx];
    const int wp = w.wpar;
    const int n = m.wspk_count[wp];
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    // the other parity's list was consumed by the previous window's delivery
    // and is refilled only by the next window: clear it for that window
    if (blockIdx.x == 0 && threadIdx.x == 0) m.wspk_count[wp ^ 1] = 0;
    for (int e = warp; e < n; e += nwarps) {
        int src = m.wspk_src[wp][e];
        int log_step = m.wspk_step[wp][e];
        uint32_t bit = 1u << (uint32_t)(log_step - w.step0);
        int64_t f0 = m.fan0[src], f1 = m.fan0[src + 1];
        for (int64_t f = f0 + lane; f < f1; f += 32) atomicOr(&m.sy_mask[m.fan_syn[f]], bit);
        if (lane == 0) {
            unsigned long long slot = atomicAdd(m.log_count, 1ull);
            if ((int64_t)slot < m.log_cap) {
                m.log_src[slot] = src;
                m.log_step[slot] = log_step;
            } else {
                atomicOr(m.status, ST_LOG_OVERFLOW);
            }
        }
    }
}

// Windowed path: one CTA advances one group of cells K steps.  Within a
// window no cell reads another cell's state: the only coupling is through
// synaptic triggers, and every connection delay is >= K * dt, so a spike
// emitted inside the window cannot fire a synapse before the window ends.
// Its trigger bits are delivered after the window (k_deliver_t) and replayed
// in order at the start of the next one (replay_mask), which reproduces the
// step-by-step pending-spike decisions exactly.  The group's membrane
// potentials, Hines diagonal and off-diagonals and per-target input currents
// live in shared memory for the whole window (gcap targets per group).
template <bool SMEM>
__global__ void __launch_bounds__(256) k_window_t(DevModel m, const WindowArgs *tab, const int *base, int idx, int gcap) {
    extern __shared__ float sm[];
    const WindowArgs w = tab[*base + idx];
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    for (int g = blockIdx.x; g < m.n_group; g += gridDim.x) {
        const int t0 = m.g_t0[g], n = m.g_t1[g] - t0;
        float *V[2], *D, *U, *L, *sIin, *sGin, *sIsyn, *sGsyn;
        int b0;
        if (SMEM) {
            V[0] = sm; V[1] = sm + gcap; D = sm + 2 * gcap; U = sm + 3 * gcap; L = sm + 4 * gcap;
            sIin = sm + 5 * gcap; sGin = sm + 6 * gcap; sIsyn = sm + 7 * gcap; sGsyn = sm + 8 * gcap;
            b0 = t0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                V[w.par][i] = m.v[w.par][t0 + i];
                U[i] = m.c_u[t0 + i];
                L[i] = m.c_l[t0 + i];
                sIin[i] = 0.f; sGin[i] = 0.f; sIsyn[i] = 0.f; sGsyn[i] = 0.f;
            }
            __syncthreads();
        } else {
            V[0] = m.v[0]; V[1] = m.v[1]; D = m.diag; U = const_cast<float *>(m.c_u); L = const_cast<float *>(m.c_l);
            sIin = m.in_I; sGin = m.in_G; sIsyn = m.syn_I; sGsyn = m.syn_G;
            b0 = 0;
        }
        int par = w.par;
        double time = w.t0;
        for (int k = 0; k < w.K; k++) {
            const int64_t step = w.step0 + k;
            const bool init = step <= 0;
            const float t = (float)time;
            float *vin = V[par], *vout = V[par ^ 1];
            for (int ii = m.g_i0[g] + warp; ii < m.g_i1[g]; ii += nwarps) {
                int tg = m.in_tgt[ii];
                float Iin, Gin, Isyn, Gsyn;
                inputs_warp(m, tg, w, step, t, k == 0, vin[tg - b0], Iin, Gin, Isyn, Gsyn);
                if ((threadIdx.x & 31) == 0) {
                    sIin[tg - b0] = Iin; sGin[tg - b0] = Gin; sIsyn[tg - b0] = Isyn; sGsyn[tg - b0] = Gsyn;
                }
            }
            __syncthreads();
            const int nround = (n + 31) & ~31;
            for (int i = threadIdx.x; i < nround; i += blockDim.x) {
                if (i < n) {
                    int tl = t0 + i - b0;
                    target_step(m, t0 + i, init, step, vin[tl], sIin[tl], sGin[tl], sIsyn[tl], sGsyn[tl], &vout[tl],
                                &D[tl], w.wpar);
                }
            }
            __syncthreads();
            for (int f = m.g_f0[g] + warp; f < m.g_f1[g]; f += nwarps)
                hines_forest(m, f, init, step, D, vout, U, L, vin, b0, w.wpar);
            __syncthreads();
            par ^= 1;
            if (!init) time += (double)m.dt;
        }
        if (SMEM) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) m.v[par][t0 + i] = V[par][i];
            __syncthreads();
        }
    }
}

__global__ void k_bump(int *base, int by) { *base += by; }

}  // namespace eden

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
            if (t.fwd_kind[g] < 0 || t.fwd_kind[g] > 2 || t.rev_kind[g] < 0 || t.rev_kind[g] > 2)
                return ctx->fail(EDEN_GPU_E_INVALID, "channel type %d gate %d: rate kind", k, g);
        }
    }
    int64_t nt = (int64_t)m->n_comp + m->n_izh;
    if (nt == 0) return ctx->fail(EDEN_GPU_E_INVALID, "empty network");
    if (m->n_src != m->n_phys + m->n_izh)
        return ctx->fail(EDEN_GPU_E_INVALID, "need one spike source per cell (n_src %d, cells %d)", m->n_src,
                         m->n_phys + m->n_izh);
    for (int s = 0; s < m->n_src; s++)
        if (m->src_target[s] < 0 || m->src_target[s] >= nt) return ctx->fail(EDEN_GPU_E_INVALID, "source %d: bad target", s);
    for (int k = 0; k < m->n_syn_types; k++) {
        const EdenGpuSynapseType &t = m->syn_types[k];
        if (t.kind != EDEN_SYN_EXPONE && t.kind != EDEN_SYN_EXPTWO) return ctx->fail(EDEN_GPU_E_INVALID, "synapse type kind");
        if (!finite_pos(t.tau_decay) || (t.kind == EDEN_SYN_EXPTWO && !finite_pos(t.tau_rise)))
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
    for (int64_t k = 0; k < m->n_pulse; k++)
        if (m->pulse_target[k] < 0 || m->pulse_target[k] >= nt)
            return ctx->fail(EDEN_GPU_E_INVALID, "pulse %lld: bad target", (long long)k);
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" int edenGpuAbiVersion(void) { return EDEN_GPU_ABI_VERSION; }

extern "C" const char *edenGpuLastError(EdenGpuCtx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" void edenGpuDestroy(EdenGpuCtx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    for (void *p : ctx->allocs) cudaFree(p);
    if (ctx->h_wtab) cudaFreeHost(ctx->h_wtab);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static int build_and_upload(EdenGpuCtx *ctx, const EdenGpuModel *m, const EdenGpuOptions *opt) {
    const int n_comp = m->n_comp, n_izh = m->n_izh, n_phys = m->n_phys;
    const int nt = n_comp + n_izh;
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
    for (int64_t k = 0; k < m->n_pulse; k++) n_in_user[m->pulse_target[k]]++;
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
        } else {
            c = 6.0 + n_in_user[n_comp + cell_izh[g]];
        }
        cost[g] = c;
        total += c;
    }

    // ---- groups: contiguous cells, balanced work, at most gcap targets
    // gcap is sized so that four CTAs fit an SM's shared memory
    const int smem_per_sm = ctx->smem_per_sm;
    int gcap = std::max(256, std::min(4096, (smem_per_sm / 4) / (9 * (int)sizeof(float))));
    gcap = std::max(gcap, max_cell);
    ctx->smem_window = (size_t)gcap * 9 * sizeof(float) <= (size_t)ctx->smem_optin;
    int cells_per_block = opt ? opt->cells_per_block : 0;
    int want_groups = std::max(1, ctx->n_sm * 4 * 2);
    std::vector<std::pair<int, int>> groups;  // [cell0, cell1)
    {
        double target = total / want_groups;
        int g = 0;
        while (g < n_cells) {
            int start = g, ntg = 0;
            double acc = 0;
            if (cells_per_block > 0) {
                while (g < n_cells && g - start < cells_per_block && (ntg + cell_n[g] <= gcap || g == start))
                    ntg += cell_n[g++];
            } else {
                while (g < n_cells && (acc < target || g == start) && (ntg + cell_n[g] <= gcap || g == start)) {
                    acc += cost[g];
                    ntg += cell_n[g++];
                }
            }
            groups.push_back({start, g});
        }
    }

    // ---- internal order: per group, per forest a joint breadth-first order
    std::vector<int32_t> u2i(nt, -1), i2u(nt, -1);
    std::vector<int32_t> c_parent(nt, -1), c_child0(nt, 0), c_nchild(nt, 0), t_izh(nt, -1);
    std::vector<float> c_u(nt, 0.f), c_l(nt, 0.f);
    std::vector<int32_t> fo_t0, fo_t1, fo_l0, fo_nlev, lvl;
    std::vector<int32_t> g_t0, g_t1, g_f0, g_f1;
    const int warps_per_block = kThreads / 32;
    int next = 0;
    int max_forest = 1;
    std::vector<int> coff, kids, fill;
    for (auto &gr : groups) {
        g_t0.push_back(next);
        g_f0.push_back((int)fo_t0.size());
        std::vector<int> phys;
        for (int g = gr.first; g < gr.second; g++)
            if (cell_phys[g] >= 0) phys.push_back(g);
        // split the group's physical cells into up to warps_per_block forests of similar size
        int64_t comps = 0;
        for (int g : phys) comps += cell_n[g];
        int nf = std::min<int>(warps_per_block, (int)phys.size());
        size_t pi = 0;
        int64_t acc = 0;
        for (int f = 0; f < nf; f++) {
            int64_t want = (comps * (f + 1)) / nf;
            const size_t later = (size_t)(nf - 1 - f);
            std::vector<int> fc;
            while (pi < phys.size()) {
                if (!fc.empty() && phys.size() - pi <= later) break;          // leave a cell per later forest
                if (!fc.empty() && f < nf - 1 && acc + cell_n[phys[pi]] > want) break;
                acc += cell_n[phys[pi]];
                fc.push_back(phys[pi++]);
            }
            if (fc.empty()) continue;
            // joint BFS over the forest's cells
            struct Node { int cell_base; int local; int depth; };
            std::vector<Node> q;
            for (int g : fc) q.push_back({m->phys_comp_off[cell_phys[g]], 0, 0});
            int f_t0 = next;
            fo_t0.push_back(f_t0);
            fo_l0.push_back((int)lvl.size());
            lvl.push_back(f_t0);
            int depth = 0;
            // children lists of each cell, built on first visit
            std::vector<std::vector<int>> cell_kids(fc.size());
            std::vector<int> cell_of_base;
            for (size_t ci = 0; ci < fc.size(); ci++) {
                int pcell = cell_phys[fc[ci]];
                int a = m->phys_comp_off[pcell], b = m->phys_comp_off[pcell + 1], n = b - a;
                coff.assign(n + 1, 0);
                for (int i = 1; i < n; i++) coff[m->comp_parent[a + i] + 1]++;
                for (int i = 0; i < n; i++) coff[i + 1] += coff[i];
                kids.assign(n > 1 ? n - 1 : 1, 0);
                fill.assign(n, 0);
                for (int i = 1; i < n; i++) {
                    int p = m->comp_parent[a + i];
                    kids[coff[p] + fill[p]++] = i;
                }
                // store as flattened: [coff (n+1)] [kids (n-1)]
                std::vector<int> &ck = cell_kids[ci];
                ck.assign(coff.begin(), coff.end());
                ck.insert(ck.end(), kids.begin(), kids.begin() + std::max(0, n - 1));
            }
            std::vector<int> node_cell;  // forest cell index of each queued node
            for (size_t ci = 0; ci < fc.size(); ci++) node_cell.push_back((int)ci);
            for (size_t h = 0; h < q.size(); h++) {
                Node u = q[h];
                int ci = node_cell[h];
                if (u.depth != depth) {
                    depth = u.depth;
                    lvl.push_back(f_t0 + (int)h);
                }
                int it = f_t0 + (int)h;
                int ut = u.cell_base + u.local;
                u2i[ut] = it;
                i2u[it] = ut;
                const std::vector<int> &ck = cell_kids[ci];
                int pcell = cell_phys[fc[ci]];
                int n = m->phys_comp_off[pcell + 1] - m->phys_comp_off[pcell];
                int k0 = ck[u.local], k1 = ck[u.local + 1];
                c_nchild[it] = k1 - k0;
                c_child0[it] = k1 > k0 ? f_t0 + (int)q.size() : 0;
                for (int k = k0; k < k1; k++) {
                    q.push_back({u.cell_base, ck[n + 1 + k], u.depth + 1});
                    node_cell.push_back(ci);
                }
            }
            int fn = (int)q.size();
            lvl.push_back(f_t0 + fn);
            fo_nlev.push_back(depth + 1);
            fo_t1.push_back(f_t0 + fn);
            max_forest = std::max(max_forest, fn);
            next += fn;
        }
        // the group's izhikevich neurons follow its forests
        for (int g = gr.first; g < gr.second; g++) {
            if (cell_izh[g] < 0) continue;
            int ut = n_comp + cell_izh[g];
            u2i[ut] = next;
            i2u[next] = ut;
            t_izh[next] = cell_izh[g];
            next++;
        }
        g_t1.push_back(next);
        g_f1.push_back((int)fo_t0.size());
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
    ctx->user_to_internal = u2i;
    ctx->gcap = gcap;
    ctx->forest_cap = max_forest;
    // ---- per-target constants in internal order
    std::vector<float> c_cm(nt, 1.f), c_inv(nt, 0.f), c_area(nt, 0.f), v0(nt, 0.f);
    std::vector<int32_t> c_chan0(nt + 1, 0);
    for (int it = 0; it < nt; it++) {
        int ut = i2u[it];
        if (ut < n_comp) {
            c_cm[it] = m->comp_c[ut];
            c_inv[it] = m->comp_inv_rc[ut];
            c_area[it] = m->comp_area[ut];
            v0[it] = m->comp_v0[ut];
            c_chan0[it + 1] = m->comp_chan_off[ut + 1] - m->comp_chan_off[ut];
        } else {
            v0[it] = m->izh_params[10 * (int64_t)(ut - n_comp) + 1];
        }
    }
    for (int it = 0; it < nt; it++) c_chan0[it + 1] += c_chan0[it];
    int n_chan = c_chan0[nt];
    std::vector<int32_t> ch_type(n_chan), ch_gate0(n_chan + 1, 0);
    std::vector<float> ch_g(n_chan), ch_e(n_chan);
    for (int it = 0; it < nt; it++) {
        int ut = i2u[it];
        if (ut >= n_comp) continue;
        int o = c_chan0[it];
        for (int ch = m->comp_chan_off[ut]; ch < m->comp_chan_off[ut + 1]; ch++, o++) {
            ch_type[o] = m->chan_type[ch];
            ch_g[o] = m->chan_gbase[ch];
            ch_e[o] = m->chan_erev[ch];
        }
    }
    for (int ch = 0; ch < n_chan; ch++) ch_gate0[ch + 1] = ch_gate0[ch] + m->chan_types[ch_type[ch]].n_gates;
    int n_gate = ch_gate0[n_chan];

    // izhikevich structure of arrays
    std::vector<float> iz[10];
    for (int f = 0; f < 10; f++) {
        iz[f].resize(n_izh);
        for (int k = 0; k < n_izh; k++) iz[f][k] = m->izh_params[10 * (int64_t)k + f];
    }

    // ---- inputs sorted by internal target (then type, then input order)
    auto sort_items = [&](int64_t n, const int32_t *tgt, const int32_t *type) {
        std::vector<int64_t> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](int64_t x, int64_t y) {
            int tx = u2i[tgt[x]], ty = u2i[tgt[y]];
            if (tx != ty) return tx < ty;
            if (type) return type[x] < type[y];
            return false;
        });
        return idx;
    };
    auto offsets = [&](const std::vector<int64_t> &order, const int32_t *tgt) {
        std::vector<int64_t> off(nt + 1, 0);
        for (int64_t k : order) off[u2i[tgt[k]] + 1]++;
        for (int t = 0; t < nt; t++) off[t + 1] += off[t];
        return off;
    };
    std::vector<int64_t> qord = sort_items(m->n_pulse, m->pulse_target, nullptr);
    std::vector<int64_t> pord = sort_items(m->n_pois, m->pois_target, m->pois_type);
    std::vector<int64_t> sord = sort_items(m->n_syn, m->syn_target, m->syn_type);
    std::vector<int64_t> qoff = offsets(qord, m->pulse_target);
    std::vector<int64_t> poff = offsets(pord, m->pois_target);
    std::vector<int64_t> soff = offsets(sord, m->syn_target);
    std::vector<int32_t> t_pulse0(nt + 1), t_pois0(nt + 1);
    for (int t = 0; t <= nt; t++) {
        t_pulse0[t] = (int32_t)qoff[t];
        t_pois0[t] = (int32_t)poff[t];
    }
    std::vector<float> pu_s(m->n_pulse), pu_d(m->n_pulse), pu_a(m->n_pulse), pu_w(m->n_pulse);
    for (int64_t k = 0; k < m->n_pulse; k++) {
        int64_t o = qord[k];
        pu_s[k] = m->pulse_start[o]; pu_d[k] = m->pulse_duration[o];
        pu_a[k] = m->pulse_amplitude[o]; pu_w[k] = m->pulse_weight[o];
    }
    std::vector<float> po_rate(m->n_pois), po_w(m->n_pois);
    std::vector<int32_t> po_seed(m->n_pois), po_inst(m->n_pois), po_tgt(m->n_pois);
    std::vector<uint8_t> po_type(m->n_pois);
    for (int64_t k = 0; k < m->n_pois; k++) {
        int64_t o = pord[k];
        po_rate[k] = m->pois_rate[o]; po_w[k] = m->pois_weight[o];
        po_seed[k] = m->src_cell_seed[m->pois_src[o]];
        po_inst[k] = m->pois_instance[o];
        po_type[k] = (uint8_t)m->pois_type[o];
        po_tgt[k] = u2i[m->pois_target[o]];
    }
    const int64_t ns = m->n_syn;
    ctx->n_syn = ns;
    std::vector<float> sy_w(ns), sy_d(ns), sy_pend(ns, -INFINITY);
    std::vector<uint8_t> sy_type(ns);
    std::vector<int32_t> sy_tgt(ns);
    ctx->syn_internal_of_user.assign(ns, 0);
    float min_delay = INFINITY;
    for (int64_t k = 0; k < ns; k++) {
        int64_t o = sord[k];
        sy_w[k] = m->syn_weight[o]; sy_d[k] = m->syn_delay[o];
        sy_type[k] = (uint8_t)m->syn_type[o];
        sy_tgt[k] = u2i[m->syn_target[o]];
        ctx->syn_internal_of_user[o] = k;
        min_delay = std::min(min_delay, m->syn_delay[o]);
    }
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
        t_src[u2i[m->src_target[s]]] = s;
        src_thr[s] = m->src_threshold[s];
    }

    // ---- window length: every delay must cover the window (see k_window)
    int kmax = 31;
    if (ns > 0) {
        double dsteps = std::floor((double)min_delay / (double)dt);
        kmax = (int)std::max(1.0, std::min(31.0, dsteps));
    }
    ctx->mode = opt ? opt->mode : EDEN_MODE_PLAIN;
    int kreq = (opt && opt->steps_per_launch > 0) ? opt->steps_per_launch : kmax;
    ctx->K = ctx->mode == EDEN_MODE_BATCHED ? std::max(1, std::min(kreq, kmax)) : 1;

    // ---- recording
    int32_t n_trace = opt ? opt->n_trace : 0;
    std::vector<int32_t> t_trace0(nt + 1, 0), trace_col(n_trace);
    {
        std::vector<std::vector<int>> cols(nt);
        for (int j = 0; j < n_trace; j++) {
            int ut = opt->trace_target[j];
            if (ut < 0 || ut >= nt) return ctx->fail(EDEN_GPU_E_INVALID, "trace column %d: bad target", j);
            cols[u2i[ut]].push_back(j);
        }
        for (int t = 0; t < nt; t++) t_trace0[t + 1] = t_trace0[t] + (int)cols[t].size();
        for (int t = 0; t < nt; t++)
            for (size_t k = 0; k < cols[t].size(); k++) trace_col[t_trace0[t] + k] = cols[t][k];
    }
    ctx->n_trace = n_trace;
    ctx->trace_cap = (opt && opt->record_capacity_steps > 0) ? opt->record_capacity_steps : 4096;
    int64_t log_cap = (opt && opt->spike_capacity > 0) ? opt->spike_capacity : (int64_t)1 << 22;

    // ---- upload
    DevModel &d = ctx->d;
    // targets with any input, in internal order; each group's are contiguous
    std::vector<int32_t> in_tgt, g_i0, g_i1;
    {
        size_t gi = 0;
        for (size_t gg = 0; gg < g_t0.size(); gg++) {
            g_i0.push_back((int)in_tgt.size());
            for (int t = g_t0[gg]; t < g_t1[gg]; t++)
                if (t_pulse0[t + 1] > t_pulse0[t] || t_pois0[t + 1] > t_pois0[t] || soff[t + 1] > soff[t])
                    in_tgt.push_back(t);
            g_i1.push_back((int)in_tgt.size());
            gi++;
        }
    }
    d.n_target = nt; d.n_src = m->n_src; d.n_group = (int)g_t0.size(); d.n_forest = (int)fo_t0.size();
    d.n_in = (int)in_tgt.size();
    d.n_syn = ns; d.n_pois = m->n_pois; d.dt = dt;
    TRY(upload_vec(ctx, &d.v[0], v0));
    TRY(upload_vec(ctx, &d.v[1], v0));
    TRY(upload(ctx, &d.diag, (const float *)nullptr, nt));
    TRY(upload_c(ctx, &d.c_cm, c_cm)); TRY(upload_c(ctx, &d.c_inv_rc, c_inv)); TRY(upload_c(ctx, &d.c_area, c_area));
    TRY(upload_c(ctx, &d.c_u, c_u)); TRY(upload_c(ctx, &d.c_l, c_l));
    TRY(upload_c(ctx, &d.c_nchild, c_nchild)); TRY(upload_c(ctx, &d.c_child0, c_child0));
    TRY(upload_c(ctx, &d.c_parent, c_parent)); TRY(upload_c(ctx, &d.t_izh, t_izh));
    TRY(upload_c(ctx, &d.fo_t0, fo_t0)); TRY(upload_c(ctx, &d.fo_t1, fo_t1)); TRY(upload_c(ctx, &d.fo_l0, fo_l0));
    TRY(upload_c(ctx, &d.fo_nlev, fo_nlev)); TRY(upload_c(ctx, &d.lvl, lvl));
    TRY(upload_c(ctx, &d.in_tgt, in_tgt));
    TRY(upload(ctx, &d.in_I, (const float *)nullptr, (size_t)nt));
    TRY(upload(ctx, &d.in_G, (const float *)nullptr, (size_t)nt));
    TRY(upload(ctx, &d.syn_I, (const float *)nullptr, (size_t)nt));
    TRY(upload(ctx, &d.syn_G, (const float *)nullptr, (size_t)nt));
    TRY(upload_c(ctx, &d.c_chan0, c_chan0)); TRY(upload_c(ctx, &d.ch_type, ch_type));
    TRY(upload_c(ctx, &d.ch_gate0, ch_gate0)); TRY(upload_c(ctx, &d.ch_gbase, ch_g)); TRY(upload_c(ctx, &d.ch_erev, ch_e));
    TRY(upload(ctx, &d.gate, (const float *)nullptr, (size_t)n_gate));
    const float **izp[10] = {&d.iz_C, &d.iz_v0, &d.iz_k, &d.iz_vr, &d.iz_vt, &d.iz_vpeak, &d.iz_a, &d.iz_b, &d.iz_c, &d.iz_d};
    for (int f = 0; f < 10; f++) TRY(upload_c(ctx, izp[f], iz[f]));
    TRY(upload(ctx, &d.iz_u, (const float *)nullptr, (size_t)n_izh));
    TRY(upload_c(ctx, &d.t_pulse0, t_pulse0)); TRY(upload_c(ctx, &d.t_pois0, t_pois0));
    TRY(upload_c(ctx, &d.t_syn0, soff));
    TRY(upload_c(ctx, &d.pu_start, pu_s)); TRY(upload_c(ctx, &d.pu_dur, pu_d));
    TRY(upload_c(ctx, &d.pu_amp, pu_a)); TRY(upload_c(ctx, &d.pu_w, pu_w));
    TRY(upload(ctx, &d.po_ts, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_isi, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_a, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload(ctx, &d.po_b, (const float *)nullptr, (size_t)m->n_pois));
    TRY(upload_c(ctx, &d.po_rate, po_rate)); TRY(upload_c(ctx, &d.po_w, po_w));
    TRY(upload_c(ctx, &d.po_seed, po_seed)); TRY(upload_c(ctx, &d.po_inst, po_inst));
    TRY(upload_c(ctx, &d.po_type, po_type));
    TRY(upload(ctx, &d.sy_a, (const float *)nullptr, (size_t)ns));
    TRY(upload(ctx, &d.sy_b, (const float *)nullptr, (size_t)ns));
    TRY(upload_vec(ctx, &d.sy_pend, sy_pend));
    TRY(upload(ctx, &d.sy_mask, (const uint32_t *)nullptr, (size_t)ns));
    TRY(upload_c(ctx, &d.sy_w, sy_w)); TRY(upload_c(ctx, &d.sy_delay, sy_d));
    TRY(upload_c(ctx, &d.sy_type, sy_type));
    TRY(upload_c(ctx, &d.t_src, t_src)); TRY(upload_c(ctx, &d.src_thr, src_thr));
    TRY(upload_c(ctx, &d.fan0, fan0)); TRY(upload_c(ctx, &d.fan_syn, fan_syn));
    // a source spikes at most once per step: a window list never exceeds n_src * K
    size_t wcap = (size_t)m->n_src * (size_t)std::max(ctx->K, 4) + 32;
    for (int b = 0; b < 2; b++) {
        TRY(upload(ctx, &d.wspk_src[b], (const int32_t *)nullptr, wcap));
        TRY(upload(ctx, &d.wspk_step[b], (const int32_t *)nullptr, wcap));
    }
    TRY(upload(ctx, &d.wspk_count, (const int32_t *)nullptr, 2));
    TRY(upload(ctx, &d.log_src, (const int32_t *)nullptr, (size_t)log_cap));
    TRY(upload(ctx, &d.log_step, (const int64_t *)nullptr, (size_t)log_cap));
    TRY(upload(ctx, &d.log_count, (const unsigned long long *)nullptr, 1));
    d.log_cap = log_cap;
    TRY(upload_c(ctx, &d.t_trace0, t_trace0)); TRY(upload_c(ctx, &d.trace_col, trace_col));
    d.n_trace = n_trace;
    TRY(upload(ctx, &d.trace_buf, (const float *)nullptr, (size_t)ctx->trace_cap * (size_t)std::max(n_trace, 1)));
    d.trace_cap = ctx->trace_cap;
    TRY(upload_c(ctx, &d.g_t0, g_t0)); TRY(upload_c(ctx, &d.g_t1, g_t1));
    TRY(upload_c(ctx, &d.g_f0, g_f0)); TRY(upload_c(ctx, &d.g_f1, g_f1));
    TRY(upload_c(ctx, &d.g_i0, g_i0)); TRY(upload_c(ctx, &d.g_i1, g_i1));
    TRY(upload(ctx, &d.status, (const int32_t *)nullptr, 1));
    TRY(upload(ctx, &ctx->d_base, (const int *)nullptr, 1));
    TRY(upload(ctx, &ctx->d_zero, (const int *)nullptr, 1));

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
        }
    }
    SynTypeDev st[kMaxSynTypes];
    memset(st, 0, sizeof(st));
    for (int k = 0; k < m->n_syn_types; k++) {
        const EdenGpuSynapseType &s = m->syn_types[k];
        st[k].kind = s.kind; st[k].gbase = s.gbase; st[k].erev = s.erev;
        st[k].tau_decay = s.tau_decay; st[k].tau_rise = s.tau_rise;
        st[k].wf_w = s.weight_prop * s.waveform_factor;
    }
    CUDA_TRY(ctx, cudaMemcpyToSymbol(c_chan_types, ct, sizeof(ct)));
    CUDA_TRY(ctx, cudaMemcpyToSymbol(c_syn_types, st, sizeof(st)));

    // ---- launch shapes
    auto blocks_for = [&](int64_t n) {
        int64_t b = (n + kThreads - 1) / kThreads;
        return (int)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ctx->n_sm * 32));
    };
    ctx->grid_inputs = blocks_for((int64_t)d.n_in * 32);
    ctx->grid_targets = blocks_for(nt);
    ctx->grid_hines = blocks_for((int64_t)d.n_forest * 32);
    ctx->grid_deliver = ctx->n_sm * 4;
    ctx->grid_window = d.n_group;
    // per-step Hines: each warp stages a forest of up to forest_cap compartments (5 arrays)
    ctx->smem_hines = (size_t)warps_per_block * 5 * ctx->forest_cap * sizeof(float);
    if (ctx->smem_hines > (size_t)ctx->smem_optin) {
        ctx->forest_cap = (int)(ctx->smem_optin / (warps_per_block * 5 * sizeof(float)));
        ctx->smem_hines = (size_t)warps_per_block * 5 * ctx->forest_cap * sizeof(float);
    }
    ctx->smem_win = ctx->smem_window ? (size_t)ctx->gcap * 9 * sizeof(float) : 0;
    CUDA_TRY(ctx, cudaFuncSetAttribute(k_hines_t, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->smem_hines));
    if (ctx->smem_window)
        CUDA_TRY(ctx, cudaFuncSetAttribute(k_window_t<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)ctx->smem_win));
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
    if (ctx->h_wtab) cudaFreeHost(ctx->h_wtab);
    if (ctx->d_wtab) {
        cudaFree(ctx->d_wtab);
        ctx->allocs.erase(std::remove(ctx->allocs.begin(), ctx->allocs.end(), (void *)ctx->d_wtab), ctx->allocs.end());
    }
    CUDA_TRY(ctx, cudaMallocHost(&ctx->h_wtab, sizeof(WindowArgs) * cap));
    void *p = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&p, sizeof(WindowArgs) * cap));
    ctx->allocs.push_back(p);
    ctx->d_wtab = (WindowArgs *)p;
    ctx->wtab_cap = cap;
    return 0;
}

// Launch the kernels of window `idx` of the current table; returns launches.
static int launch_window(EdenGpuCtx *ctx, const int *base, int idx, int K) {
    DevModel &d = ctx->d;
    cudaStream_t s = ctx->stream;
    if (ctx->mode == EDEN_MODE_BATCHED) {
        if (ctx->smem_window)
            k_window_t<true><<<ctx->grid_window, kThreads, ctx->smem_win, s>>>(d, ctx->d_wtab, base, idx, ctx->gcap);
        else
            k_window_t<false><<<ctx->grid_window, kThreads, 0, s>>>(d, ctx->d_wtab, base, idx, ctx->gcap);
        k_deliver_t<<<ctx->grid_deliver, kThreads, 0, s>>>(d, ctx->d_wtab, base, idx);
        return 2;
    }
    (void)K;
    k_inputs_t<<<ctx->grid_inputs, kThreads, 0, s>>>(d, ctx->d_wtab, base, idx);
    k_targets_t<<<ctx->grid_targets, kThreads, 0, s>>>(d, ctx->d_wtab, base, idx);
    k_hines_t<<<ctx->grid_hines, kThreads, ctx->smem_hines, s>>>(d, ctx->d_wtab, base, idx, ctx->forest_cap);
    k_deliver_t<<<ctx->grid_deliver, kThreads, 0, s>>>(d, ctx->d_wtab, base, idx);
    return 4;
}

extern "C" int edenGpuRun(EdenGpuCtx *ctx, int64_t first_step, int64_t n_steps) {
    if (!ctx) return EDEN_GPU_E_INVALID;
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
    for (size_t i = 0; i < wins.size(); i++) {
        WindowArgs &w = ctx->h_wtab[i];
        w.step0 = wins[i].step0;
        w.K = wins[i].K;
        w.Kprev = ctx->Kprev;
        w.t0 = ctx->time;
        w.t_prev0 = ctx->t_prev0;
        w.par = ctx->par;
        w.wpar = ctx->wpar;
        if (w.step0 > 0) {
            ctx->t_prev0 = ctx->time;
            ctx->Kprev = w.K;
            for (int k = 0; k < w.K; k++) ctx->time += (double)ctx->d.dt;
        }
        ctx->par ^= (w.K & 1);
        ctx->wpar ^= 1;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_wtab, ctx->h_wtab, sizeof(WindowArgs) * wins.size(), cudaMemcpyHostToDevice,
                                  ctx->stream));
    CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_base, 0, sizeof(int), ctx->stream));
    CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    int64_t launches = 0;
    size_t i = 0;
    // graph replay for full chunks of regular windows (batched mode)
    if (ctx->mode == EDEN_MODE_BATCHED) {
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
            CUDA_TRY(ctx, cudaGraphLaunch(ctx->graph, ctx->stream));
            launches += kGraphWindows * 2 + 1;
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
    ctx->next_step = last + 1;
    int status = 0;
    CUDA_TRY(ctx, cudaMemcpy(&status, ctx->d.status, sizeof(int), cudaMemcpyDeviceToHost));
    ctx->sticky_status |= status;
    if (status & ST_LOG_OVERFLOW) return ctx->fail(EDEN_GPU_E_RANGE, "spike log overflow; fetch records more often");
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
    std::vector<float> tmp(std::max<int64_t>(n, 1));
    float *outs[3] = {pending_us, state_a, state_b};
    float *srcs[3] = {ctx->d.sy_pend, ctx->d.sy_a, ctx->d.sy_b};
    for (int k = 0; k < 3; k++) {
        if (!outs[k] || n == 0) continue;
        CUDA_TRY(ctx, cudaMemcpy(tmp.data(), srcs[k], sizeof(float) * n, cudaMemcpyDeviceToHost));
        for (int64_t u = 0; u < n; u++) outs[k][u] = tmp[ctx->syn_internal_of_user[u]];
    }
    return 0;
}
