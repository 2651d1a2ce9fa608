/*
 * eden_port_gpu.cu — the C restatement of the reference loop
 * (oracle/port/eden_port.c) compiled for the GPU in double precision: the
 * FP64 GPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: a checker for the single-precision GPU path at
 * sizes and lengths the host cores cannot reach in reasonable time.  It is
 * the same source as the CPU restatement, built with EDEN_PORT_DOUBLE and
 * run one thread per cell per step (the reference's OpenMP loop over work
 * items, eden/Eden.cpp:11846-11869), so it inherits that restatement's
 * citations and its pinning against the reference's outputs; the product
 * never links or calls it.
 *
 * Per step: an output kernel records the trajectory columns and logs the
 * spikes flagged in the "now" buffers (eden/Eden.cpp:11555-11635), then one
 * thread per cell runs phys_cell_step / izh_step, writing the "next"
 * buffers; the host adds dt to the double time and swaps the buffers.
 */
#define EDEN_PORT_DOUBLE
#include "../port/eden_port.c"

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace {

struct Gpu {
    std::vector<void *> allocs;
    cudaError_t err = cudaSuccess;

    template <typename T>
    T *copy(const T *src, size_t n) {
        void *p = nullptr;
        if (err != cudaSuccess) return nullptr;
        err = cudaMalloc(&p, (n > 0 ? n : 1) * sizeof(T));
        if (err != cudaSuccess) return nullptr;
        allocs.push_back(p);
        if (src && n) err = cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice);
        return static_cast<T *>(p);
    }
    template <typename T>
    T *zeros(size_t n) {
        T *p = copy<T>(nullptr, n);
        if (p) err = cudaMemset(p, 0, (n > 0 ? n : 1) * sizeof(T));
        return p;
    }
    ~Gpu() {
        for (void *p : allocs) cudaFree(p);
    }
};

__global__ void k_output(Port P, int cur, int64_t step, int32_t n_trace, const int32_t *tt, double *trace,
                         int64_t cap, int32_t *log_src, int64_t *log_step, unsigned long long *log_n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_trace) trace[(step - 1) * n_trace + i] = tt[i] >= 0 ? P.v[cur][tt[i]] : P.gate[cur][-2 - (int64_t)tt[i]];
    if (i < P.m->n_src && P.spiked[cur][i]) {
        const unsigned long long k = atomicAdd(log_n, 1ull);
        if ((int64_t)k < cap) {
            log_src[k] = (int32_t)i;
            log_step[k] = step;
        }
        P.spiked[cur][i] = 0;
    }
}

__global__ void k_ext(Port P, int nxt, const int32_t *ext_src, int64_t e0, int64_t e1) {
    const int64_t e = e0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < e1) send_spike(&P, nxt, ext_src[e]);
}

__global__ void k_items(Port P, int cur, int init, double t, double dt, int64_t step, int32_t n_phys, int32_t n_items) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= n_items) return;
    if (item < n_phys)
        phys_cell_step(&P, cur, item, init, t, dt, step);
    else
        izh_step(&P, cur, item - n_phys, init, t, dt, step);
}

}  // namespace

/*
 * As eden_port_run, in double precision on GPU `device`: records V of
 * `trace_target` (double, [n_steps][n_trace]) and the spikes (source,
 * logging step), in step order and by source within a step.
 */
extern "C" int eden_port_gpu_run(const EdenGpuModel *m, int64_t n_steps, int32_t n_trace,
                                 const int32_t *trace_target, double *trace, int64_t spike_cap,
                                 int32_t *spike_src, int64_t *spike_step, int64_t *n_spikes, int32_t device) {
    if (!m || m->abi_version != EDEN_GPU_ABI_VERSION) return EDEN_GPU_E_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return EDEN_GPU_E_NODEVICE;
    Port H;
    port_setup(&H, m);
    const int64_t nt = H.n_target;
    const int64_t n_chan = m->comp_chan_off[m->n_comp];
    const int64_t n_gate = H.gate_off[n_chan];
    const int64_t ns = m->n_syn, np = m->n_pois;
    int rc = 0;
    {
        Gpu g;
        // the model, with device arrays
        EdenGpuModel dm = *m;
        dm.phys_comp_off = g.copy(m->phys_comp_off, (size_t)m->n_phys + 1);
        dm.comp_parent = g.copy(m->comp_parent, (size_t)m->n_comp);
        dm.comp_c = g.copy(m->comp_c, (size_t)m->n_comp);
        dm.comp_r_axial = g.copy(m->comp_r_axial, (size_t)m->n_comp);
        dm.comp_area = g.copy(m->comp_area, (size_t)m->n_comp);
        dm.comp_inv_rc = g.copy(m->comp_inv_rc, (size_t)m->n_comp);
        dm.comp_v0 = g.copy(m->comp_v0, (size_t)m->n_comp);
        dm.chan_types = g.copy(m->chan_types, (size_t)m->n_chan_types);
        dm.comp_chan_off = g.copy(m->comp_chan_off, (size_t)m->n_comp + 1);
        dm.chan_type = g.copy(m->chan_type, (size_t)n_chan);
        dm.chan_gbase = g.copy(m->chan_gbase, (size_t)n_chan);
        dm.chan_erev = g.copy(m->chan_erev, (size_t)n_chan);
        dm.izh_params = g.copy(m->izh_params, (size_t)m->n_izh * EDEN_POINT_PARAMS);
        dm.izh_kind = m->izh_kind ? g.copy(m->izh_kind, (size_t)m->n_izh) : nullptr;
        dm.src_target = g.copy(m->src_target, (size_t)m->n_src);
        dm.src_threshold = g.copy(m->src_threshold, (size_t)m->n_src);
        dm.src_cell_seed = g.copy(m->src_cell_seed, (size_t)m->n_src);
        dm.syn_types = g.copy(m->syn_types, (size_t)m->n_syn_types);
        dm.syn_target = g.copy(m->syn_target, (size_t)ns);
        dm.syn_type = g.copy(m->syn_type, (size_t)ns);
        dm.syn_src = g.copy(m->syn_src, (size_t)ns);
        dm.syn_weight = g.copy(m->syn_weight, (size_t)ns);
        dm.syn_delay = g.copy(m->syn_delay, (size_t)ns);
        dm.pois_target = g.copy(m->pois_target, (size_t)np);
        dm.pois_type = g.copy(m->pois_type, (size_t)np);
        dm.pois_rate = g.copy(m->pois_rate, (size_t)np);
        dm.pois_weight = g.copy(m->pois_weight, (size_t)np);
        dm.pois_src = g.copy(m->pois_src, (size_t)np);
        dm.pois_instance = g.copy(m->pois_instance, (size_t)np);
        dm.pulse_target = g.copy(m->pulse_target, (size_t)m->n_pulse);
        dm.pulse_start = g.copy(m->pulse_start, (size_t)m->n_pulse);
        dm.pulse_duration = g.copy(m->pulse_duration, (size_t)m->n_pulse);
        dm.pulse_amplitude = g.copy(m->pulse_amplitude, (size_t)m->n_pulse);
        dm.pulse_weight = g.copy(m->pulse_weight, (size_t)m->n_pulse);
        dm.timed_target = g.copy(m->timed_target, (size_t)m->n_timed);
        dm.timed_type = g.copy(m->timed_type, (size_t)m->n_timed);
        dm.timed_weight = g.copy(m->timed_weight, (size_t)m->n_timed);
        dm.timed_off = g.copy(m->timed_off, (size_t)m->n_timed + 1);
        dm.timed_step = g.copy(m->timed_step, m->n_timed ? (size_t)m->timed_off[m->n_timed] : 0);
        dm.ext_src = g.copy(m->ext_src, (size_t)m->n_ext);
        dm.ext_step = g.copy(m->ext_step, (size_t)m->n_ext);
        dm.wave_target = g.copy(m->wave_target, (size_t)m->n_wave);
        dm.wave_shape = g.copy(m->wave_shape, (size_t)m->n_wave);
        dm.wave_params = g.copy(m->wave_params, (size_t)m->n_wave * EDEN_WAVE_PARAMS);
        dm.wave_weight = g.copy(m->wave_weight, (size_t)m->n_wave);
        dm.clamp_target = g.copy(m->clamp_target, (size_t)m->n_clamp);
        dm.clamp_params = g.copy(m->clamp_params, (size_t)m->n_clamp * EDEN_CLAMP_PARAMS);
        dm.clamp_weight = g.copy(m->clamp_weight, (size_t)m->n_clamp);
        dm.gap_target = g.copy(m->gap_target, (size_t)m->n_gap);
        dm.gap_peer = g.copy(m->gap_peer, (size_t)m->n_gap);
        dm.gap_conductance = g.copy(m->gap_conductance, (size_t)m->n_gap);
        dm.gap_weight = g.copy(m->gap_weight, (size_t)m->n_gap);
        dm.graded_target = g.copy(m->graded_target, (size_t)m->n_graded);
        dm.graded_peer = g.copy(m->graded_peer, (size_t)m->n_graded);
        dm.graded_params = g.copy(m->graded_params, (size_t)m->n_graded * EDEN_GRADED_PARAMS);
        dm.graded_weight = g.copy(m->graded_weight, (size_t)m->n_graded);
        dm.pois_rng_base = m->pois_rng_base ? g.copy(m->pois_rng_base, (size_t)np) : nullptr;
        // the loop's state, set up on the host
        Port D = H;
        D.m = g.copy(&dm, 1);
        for (int b = 0; b < 2; b++) {
            D.v[b] = g.copy(H.v[b], (size_t)nt + 1);
            D.gate[b] = g.copy(H.gate[b], (size_t)n_gate + 1);
            D.izh_u[b] = g.copy(H.izh_u[b], (size_t)m->n_izh + 1);
            D.izh_s[b] = g.copy(H.izh_s[b], (size_t)m->n_izh + 1);
            D.syn_a[b] = g.copy(H.syn_a[b], (size_t)ns + 1);
            D.syn_b[b] = g.copy(H.syn_b[b], (size_t)ns + 1);
            D.syn_pend[b] = g.copy(H.syn_pend[b], (size_t)ns + 1);
            D.trig[b] = g.copy(H.trig[b], (size_t)ns + 1);
            D.pois_ts[b] = g.copy(H.pois_ts[b], (size_t)np + 1);
            D.pois_isi[b] = g.copy(H.pois_isi[b], (size_t)np + 1);
            D.pois_a[b] = g.copy(H.pois_a[b], (size_t)np + 1);
            D.pois_b[b] = g.copy(H.pois_b[b], (size_t)np + 1);
            D.spiked[b] = g.copy(H.spiked[b], (size_t)m->n_src + 1);
            D.timed_a[b] = g.copy(H.timed_a[b], (size_t)m->n_timed + 1);
            D.timed_b[b] = g.copy(H.timed_b[b], (size_t)m->n_timed + 1);
            D.gr_s[b] = g.copy(H.gr_s[b], (size_t)m->n_graded + 1);
            D.syn_R[b] = g.copy(H.syn_R[b], (size_t)ns + 1);
            D.syn_U[b] = g.copy(H.syn_U[b], (size_t)ns + 1);
        }
        D.diag = g.copy(H.diag, (size_t)m->n_comp + 1);
        D.gate_off = g.copy(H.gate_off, (size_t)n_chan + 1);
        D.syn_off = g.copy(H.syn_off, (size_t)nt + 1);
        D.pois_off = g.copy(H.pois_off, (size_t)nt + 1);
        D.pulse_off = g.copy(H.pulse_off, (size_t)nt + 1);
        D.wave_off = g.copy(H.wave_off, (size_t)nt + 1);
        D.clamp_off = g.copy(H.clamp_off, (size_t)nt + 1);
        D.fan_off = g.copy(H.fan_off, (size_t)m->n_src + 1);
        D.fan_syn = g.copy(H.fan_syn, (size_t)ns + 1);
        D.order = g.copy(H.order, (size_t)m->n_comp + 1);
        D.src_of_target = g.copy(H.src_of_target, (size_t)nt + 1);
        D.syn_fire_count = g.copy(H.syn_fire_count, (size_t)ns + 1);
        D.timed_cur = g.copy(H.timed_cur, (size_t)m->n_timed + 1);
        D.timed_tgt_off = g.copy(H.timed_tgt_off, (size_t)nt + 1);
        D.timed_order = g.copy(H.timed_order, (size_t)m->n_timed + 1);
        D.gap_off = g.copy(H.gap_off, (size_t)nt + 1);
        D.gap_order = g.copy(H.gap_order, (size_t)m->n_gap + 1);
        D.gr_off = g.copy(H.gr_off, (size_t)nt + 1);
        D.gr_order = g.copy(H.gr_order, (size_t)m->n_graded + 1);
        int32_t *d_tt = g.copy(trace_target, (size_t)n_trace);
        double *d_trace = g.zeros<double>((size_t)n_steps * (size_t)(n_trace > 0 ? n_trace : 1));
        int32_t *d_lsrc = g.zeros<int32_t>((size_t)spike_cap);
        int64_t *d_lstep = g.zeros<int64_t>((size_t)spike_cap);
        unsigned long long *d_ln = g.zeros<unsigned long long>(1);
        if (g.err != cudaSuccess) {
            port_free(&H);
            return g.err == cudaErrorMemoryAllocation ? EDEN_GPU_E_NOMEM : EDEN_GPU_E_CUDA;
        }
        const int32_t n_items = m->n_phys + m->n_izh;
        const int threads = 128;
        const int grid_items = (n_items + threads - 1) / threads;
        const int64_t n_out = n_trace > m->n_src ? n_trace : m->n_src;
        const int grid_out = (int)((n_out + threads - 1) / threads);
        int cur = 0;
        int64_t ext = 0;
        double time = 0.0;
        const double dt = m->dt;
        for (int64_t step = -3; step <= n_steps; step++) {
            const int init = step <= 0;
            if (!init && grid_out > 0)
                k_output<<<grid_out, threads>>>(D, cur, step, n_trace, d_tt, d_trace, spike_cap, d_lsrc, d_lstep, d_ln);
            if (grid_items > 0) k_items<<<grid_items, threads>>>(D, cur, init, time, dt, step, m->n_phys, n_items);
            // the spike sources' events emitted this step
            int64_t e1 = ext;
            while (e1 < m->n_ext && m->ext_step[e1] <= step + 1) e1++;
            int64_t e0 = ext;
            while (e0 < e1 && m->ext_step[e0] < step + 1) e0++;
            if (e1 > e0)
                k_ext<<<(int)((e1 - e0 + threads - 1) / threads), threads>>>(D, cur ^ 1, dm.ext_src, e0, e1);
            ext = e1;
            if (!init) time += dt;
            cur ^= 1;
        }
        if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            port_free(&H);
            return EDEN_GPU_E_CUDA;
        }
        unsigned long long nl = 0;
        cudaMemcpy(&nl, d_ln, sizeof(nl), cudaMemcpyDeviceToHost);
        const int64_t keep = (int64_t)nl < spike_cap ? (int64_t)nl : spike_cap;
        if (n_trace > 0)
            cudaMemcpy(trace, d_trace, sizeof(double) * (size_t)n_steps * (size_t)n_trace, cudaMemcpyDeviceToHost);
        std::vector<int32_t> ls((size_t)keep);
        std::vector<int64_t> lk((size_t)keep);
        if (keep > 0) {
            cudaMemcpy(ls.data(), d_lsrc, sizeof(int32_t) * (size_t)keep, cudaMemcpyDeviceToHost);
            cudaMemcpy(lk.data(), d_lstep, sizeof(int64_t) * (size_t)keep, cudaMemcpyDeviceToHost);
        }
        // step order, by source within a step (the order eden_port_run logs them)
        std::vector<int64_t> idx((size_t)keep);
        for (int64_t k = 0; k < keep; k++) idx[(size_t)k] = k;
        std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) {
            return lk[(size_t)a] != lk[(size_t)b] ? lk[(size_t)a] < lk[(size_t)b] : ls[(size_t)a] < ls[(size_t)b];
        });
        for (int64_t k = 0; k < keep; k++) {
            spike_src[k] = ls[(size_t)idx[(size_t)k]];
            spike_step[k] = lk[(size_t)idx[(size_t)k]];
        }
        *n_spikes = (int64_t)nl;
        if ((int64_t)nl > spike_cap) rc = EDEN_GPU_E_RANGE;
        if (cudaGetLastError() != cudaSuccess) rc = EDEN_GPU_E_CUDA;
    }
    port_free(&H);
    return rc;
}
