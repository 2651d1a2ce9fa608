// The kernels of libeden_gpu.  This header is compiled twice: ahead of time
// into the library, and at context creation by NVRTC together with code
// generated for the model's mechanisms (EDEN_RTC, see eden_codegen.cu), the
// GPU counterpart of the per-cell-type C the reference generates and
// compiles with gcc (eden/Eden.cpp:7017-7180).
#pragma once
#include "eden_kernels.cuh"

namespace eden {

constexpr int kThreads = 256;
constexpr int kInputThreads = 128;  // k_inputs_t: four warps, each with two event tiles
constexpr int kCellThreads = 128;   // k_cells_t: four warps
constexpr int kHinesThreads = 128;  // k_hines_t: four warps, each staging one forest

}  // namespace eden

// ---------------------------------------------------------------------------
// kernels; each reads its WindowArgs from a device table so that a captured
// graph can be replayed over many windows
// ---------------------------------------------------------------------------
namespace eden {

// Phase 1 of both paths: input blocks over the window, one warp per target
// with inputs (the per-step path runs it with K = 1).  Six blocks fit an SM
// by their event tiles; the register bound lets all six run.
__global__ void __launch_bounds__(kInputThreads, 6) k_inputs_t(DevModel m, const WindowArgs *tab,
                                                             const WindowTimes *ttab, const int *base, int idx) {
    __shared__ float tiles[kInputThreads / 32][2][32 * kAccStride];
    __shared__ float tk[64];  // the window's step times, then the previous window's
    const int wi = *base + idx;
    const WindowArgs w = tab[wi];
    if (threadIdx.x < 64) tk[threadIdx.x] = threadIdx.x < 32 ? ttab[wi].tk[threadIdx.x] : ttab[wi].tprev[threadIdx.x - 32];
    __syncthreads();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    float *tileA = tiles[threadIdx.x >> 5][0], *tileB = tiles[threadIdx.x >> 5][1];
    // each warp walks its chunks with the next chunk's descriptor in flight
    int c = warp;
    int32_t info = 0;
    int64_t i0 = 0;
    if (c < m.n_chunk) { info = m.ck_info[c]; i0 = m.ck_i0[c]; }
    while (c < m.n_chunk) {
        const int cn = c + nwarps;
        int32_t info_n = 0;
        int64_t i0_n = 0;
        if (cn < m.n_chunk) { info_n = m.ck_info[cn]; i0_n = m.ck_i0[cn]; }
        chunk_window(m, c, info, i0, w, tileA, tileB, tk);
        c = cn; info = info_n; i0 = i0_n;
    }
}

// Per-step path, phase 2: one thread per target.
__global__ void __launch_bounds__(256) k_targets_t(DevModel m, const WindowArgs *tab, const WindowTimes *ttab,
                                                   const int *base, int idx) {
    const WindowArgs w = tab[*base + idx];
    const float tnow = ttab[*base + idx].tk[0];
    const bool init = w.step0 <= 0;
    const float *vin = m.v[w.par];
    float *vout = m.v[w.par ^ 1];
    const int n = m.n_target;
    const int nround = (n + 31) & ~31;  // whole warps stay converged for the spike ballot
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nround; i += gridDim.x * blockDim.x) {
        if (i < n) {
            float v = vin[i], Iin, Gin, Isyn, Gsyn;
            block_currents(m.Gp, m.t_blk0[i], m.t_blk0[i + 1], m.bk_kind, m.bk_erev, m.bk_c0, 0, v, Iin, Gin, Isyn,
                           Gsyn, m.bk_block);
            if (EDEN_KIND_GAP) Isyn += gap_current(m, i, v, vin, init);
            const float Iax = (m.fwd_euler && !init && m.t_izh[i] < 0) ? axial_current(m, i, v, vin) : 0.0f;
            target_step(m, i, init, w.step0, tnow, v, Iin, Gin, Isyn, Gsyn, &vout[i], &m.diag[i], w.wpar, Iax);
        }
    }
}

// Per-step path, phase 3: one warp per forest, staged in the warp's slice of
// shared memory when the forest has at most `cap` compartments.
__global__ void __launch_bounds__(kHinesThreads) k_hines_t(DevModel m, const WindowArgs *tab, const int *base, int idx, int cap) {
    extern __shared__ float sm[];
    const WindowArgs w = tab[*base + idx];
    const bool init = w.step0 <= 0;
    const float *vin = m.v[w.par];
    float *x = m.v[w.par ^ 1];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    // per-warp slice: D, X, U, L, V, child ends, parents, depth boundaries (cap each)
    float *sD = sm + (size_t)wib * 8 * cap, *sX = sD + cap, *sU = sX + cap, *sL = sU + cap, *sV = sL + cap;
    int32_t *sCE = (int32_t *)(sV + cap), *sP = sCE + cap, *sLV = sP + cap;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int f = warp; f < m.n_forest; f += nwarps) {
        const int c0 = m.fo_t0[f], n = m.fo_t1[f] - c0, nlev = m.fo_nlev[f];
        const int32_t *lv = m.lvl + m.fo_l0[f];
        if (m.fwd_euler) {
            // V_next is final already: only the threshold test
            hines_forest(m, true, w.step0, w.t0, m.diag, x, m.c_u, m.c_l, m.c_cend, m.c_parent, lv, nlev, vin, 0,
                         w.wpar, true);
        } else if (m.fo_f64[f]) {
            hines_forest_f64(m, init, w.step0, w.t0, m.diag, x, m.c_u, m.c_l, m.c_cend, m.c_parent, lv, nlev, vin,
                             m.dscr, m.dscr + m.n_target, w.wpar);
        } else if (n <= cap && nlev < cap) {
            for (int i = lane; i < n; i += 32) {
                sD[i] = m.diag[c0 + i]; sX[i] = x[c0 + i]; sU[i] = m.c_u[c0 + i];
                sL[i] = m.c_l[c0 + i]; sV[i] = vin[c0 + i];
                sCE[i] = m.c_cend[c0 + i] - c0; sP[i] = m.c_parent[c0 + i] - c0;
            }
            for (int i = lane; i <= nlev; i += 32) sLV[i] = lv[i] - c0;
            __syncwarp();
            hines_forest(m, init, w.step0, w.t0, sD, sX, sU, sL, sCE, sP, sLV, nlev, sV, c0, w.wpar, true);
            __syncwarp();
            for (int i = lane; i < n; i += 32) x[c0 + i] = sX[i];
            __syncwarp();
        } else {
            hines_forest(m, init, w.step0, w.t0, m.diag, x, m.c_u, m.c_l, m.c_cend, m.c_parent, lv, nlev, vin, 0, w.wpar,
                         true);
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
    // then the window's spikes of sources with no target (spike lists and
    // generators, computed in advance)
    const int n_all = n + (w.ext1 - w.ext0);
    for (int e = warp; e < n_all; e += nwarps) {
        const bool own = e < n;
        int src = own ? m.wspk_src[wp][e] : m.ext_src[w.ext0 + e - n];
        int log_step = own ? m.wspk_step[wp][e] : m.ext_step[w.ext0 + e - n];
        const double tcross = own ? m.wspk_time[wp][e] : no_time();
        uint32_t bit = 1u << (uint32_t)(log_step - w.step0);
        int64_t f0 = m.fan0[src], f1 = m.fan0[src + 1];
        for (int64_t f = f0 + lane; f < f1; f += 32) atomicOr(&m.sy_mask[m.fan_syn[f]], bit);
        if (lane == 0) {
            unsigned long long slot = atomicAdd(m.log_count, 1ull);
            if ((int64_t)slot < m.log_cap) {
                m.log_src[slot] = src;
                m.log_step[slot] = log_step;
                m.log_time[slot] = tcross;
            } else {
                atomicOr(m.status, ST_LOG_OVERFLOW);
            }
        }
    }
}

// Windowed path: every warp advances one unit (a forest of physical cells or
// a batch of izhikevich neurons) K steps on its own, synchronising only within
// the warp.  Within a window no cell reads another cell's state: the only
// coupling is through synaptic triggers, and every connection delay is
// >= K * dt, so a spike emitted inside the window cannot fire a synapse before
// the window ends.  Its trigger bits are delivered after the window
// (k_deliver_t) and replayed in order at the start of the next one
// (replay_mask), which reproduces the step-by-step pending-spike decisions
// exactly.  Synaptic conductances do not depend on V, so k_inputs_t has
// already produced them for all K steps.  Everything else a step reads is
// staged in the warp's shared-memory slice for the whole window.

// A forest unit over the window.  At the window start the unit stages its
// compartments, its non-flat compartments' descriptors, its gates with their
// parameter records, and the conductance series of its input chunks for all
// K steps (written by k_inputs_t), so that a step reads shared memory only.
// Per step: trajectory samples of the step's starting V; the non-flat
// compartments' currents (inputs, channels with the gate values before this
// step's update), diagonal and pre-update; the cable solve, which also
// applies the flat compartments' constant pre-update; gate updates from the
// starting V; threshold crossings.
__device__ __forceinline__ void forest_window(const DevModel &m, const WindowArgs &w, int u, float *S) {
    const int lane = threadIdx.x & 31;
    const int t0 = m.un_t0[u], n = m.un_t1[u] - t0, fi = m.un_f[u];
    const int ngt = m.un_ngt[u], gt0 = m.un_gt0[u];
    const int s0 = m.un_s0[u], ns = m.un_s1[u] - s0;
    const int r0 = m.un_r0[u], r1 = m.un_r1[u];
    const int nf0 = m.un_nf0[u], nf = m.un_nf1[u] - nf0;
    const int nlev = m.fo_nlev[fi], l0 = m.fo_l0[fi];
    const int ub0 = m.t_blk0[t0], nblk = m.t_blk0[t0 + n] - ub0;
    const int uc0 = m.bk_c0[ub0], nck = m.bk_c0[ub0 + nblk] - uc0;
    // compartment terms in pairs (the slice is 8-byte aligned): V and the
    // elimination factor, c_kl and the packed child range / parent / flag, U
    // and the pivot
    float2 *XR = reinterpret_cast<float2 *>(S);
    uint2 *KL = reinterpret_cast<uint2 *>(S + 2 * n);
    float2 *UP = reinterpret_cast<float2 *>(S + 4 * n);
    int32_t *NT = (int32_t *)(S + 6 * n);
    float *VO = (float *)(NT + nf), *NA = VO + nf, *NC = NA + nf, *NIR = NC + nf;
    int32_t *NB0 = (int32_t *)(NIR + nf), *NB1 = NB0 + nf, *NCH0 = NB1 + nf, *NCH1 = NCH0 + nf;
    int32_t *NSIG = NCH1 + nf;
    const int uch0 = nf > 0 ? m.nf_c0[nf0] : 0, nch = nf > 0 ? m.nf_c1[nf0 + nf - 1] - uch0 : 0;
    float *CHG = (float *)(NSIG + nf), *CHE = CHG + nch;
    int32_t *CHQ = (int32_t *)(CHE + nch), *CHI = CHQ + nch;
    float *GT = (float *)(CHI + nch);
    int32_t *GI_S = (int32_t *)(GT + ngt);
    float *GP = (float *)(GI_S + ngt);
    int32_t *LV = (int32_t *)(GP + kGateWords * ngt);
    int32_t *ST = LV + nlev + 1, *SSRC = ST + ns;
    float *STHR = (float *)(SSRC + ns);
    int32_t *BKK = (int32_t *)(STHR + ns);
    float *BKE = (float *)(BKK + nblk);
    int32_t *BKC = (int32_t *)(BKE + nblk);
    float *GS = (float *)(BKC + nblk + 1);
    // a double-precision forest's eliminated values, pivots and factors
    const bool f64 = m.fo_f64[fi] != 0;
    double *XD = reinterpret_cast<double *>((reinterpret_cast<unsigned long long>(GS + w.K * nck) + 7ull) & ~7ull);
    double *PVD = XD + n, *RTD = PVD + n;
    // ---- stage the unit
    const float *vsrc = m.v[w.par];
    const float *pv0 = f64 ? m.c_d0 : m.c_pv0;
    for (int i = lane; i < n; i += 32) {
        const int t = t0 + i;
        stage_word(&XR[i].x, &vsrc[t]); stage_word(&XR[i].y, &m.c_rt0[t]);
        stage_word(&KL[i].x, &m.c_kl[t]); stage_word(&KL[i].y, &m.c_cep[t]);
        stage_word(&UP[i].x, &m.c_u[t]); stage_word(&UP[i].y, &pv0[t]);
    }
    for (int j = lane; j < nf; j += 32) {
        const int ti = m.nf_t[nf0 + j], t = t0 + ti;
        NT[j] = ti;
        stage_word(&NA[j], &m.c_area[t]); stage_word(&NC[j], &m.c_cm[t]); stage_word(&NIR[j], &m.c_inv_rc[t]);
        NB0[j] = m.t_blk0[t] - ub0; NB1[j] = m.t_blk0[t + 1] - ub0;
        const int ch0 = m.c_chan0[t], ch1 = m.c_chan0[t + 1];
        NCH0[j] = m.nf_c0[nf0 + j] - uch0; NCH1[j] = m.nf_c1[nf0 + j] - uch0;
        stage_word(&NSIG[j], &m.nf_sig[nf0 + j]);
        // gate update items: the non-flat slot and the gate's parameter record
        for (int ch = ch0; ch < ch1; ch++) {
            const int q0 = m.ch_gate0[ch] - gt0, q1 = m.ch_gate0[ch + 1] - gt0;
            const float *src = m.gate_par + (size_t)m.ch_type[ch] * EDEN_MAX_GATES * kGateWords;
            for (int q = q0; q < q1; q++) {
                GI_S[q] = j;
                for (int k = 0; k < kGateWords; k++) stage_word(&GP[q * kGateWords + k], &src[(q - q0) * kGateWords + k]);
            }
        }
    }
    for (int c = lane; c < nch; c += 32) {
        stage_word(&CHG[c], &m.nfc_g[uch0 + c]); stage_word(&CHE[c], &m.nfc_e[uch0 + c]);
        stage_word(&CHQ[c], &m.nfc_q[uch0 + c]); stage_word(&CHI[c], &m.nfc_i[uch0 + c]);
    }
    for (int i = lane; i < ngt; i += 32) stage_word(&GT[i], &m.gate[gt0 + i]);
    for (int i = lane; i <= nlev; i += 32) {
        const int info = m.lvl_info[l0 + i];
        LV[i] = (m.lvl[l0 + i] - t0) | ((info & 0x80) ? kLvNonFlat : 0);
    }
    for (int i = lane; i < ns; i += 32) {
        stage_word(&ST[i], &m.gs_t[s0 + i]); stage_word(&SSRC[i], &m.gs_src[s0 + i]); stage_word(&STHR[i], &m.gs_thr[s0 + i]);
    }
    for (int b = lane; b <= nblk; b += 32) {
        BKC[b] = m.bk_c0[ub0 + b] - uc0;
        if (b < nblk) { stage_word(&BKK[b], &m.bk_kind[ub0 + b]); stage_word(&BKE[b], &m.bk_erev[ub0 + b]); }
    }
    for (int k = 0; k < w.K; k++)
        for (int c = lane; c < nck; c += 32) stage_word(&GS[k * nck + c], &m.Gp[(size_t)k * m.n_chunk + uc0 + c]);
    stage_wait();
    __syncwarp();
    const float dt = m.dt;
    double tstep = w.t0;  // this step's time, accumulated in double as the host does
    for (int k = 0; k < w.K; k++) {
        const int64_t step = w.step0 + k;
        const bool init = step <= 0;
        if (!init && r1 > r0) {
            // trajectory samples of this step's starting state
            const int64_t row = (step - 1) % m.trace_cap;
            for (int q = r0 + lane; q < r1; q += 32) {
                const int32_t tq = m.gr_t[q];  // a compartment, or -1 - a gate slot
                m.trace_buf[row * m.n_trace + m.gr_col[q]] = tq >= 0 ? XR[tq].x : GT[-1 - tq];
            }
        }
        __syncwarp();
        const float *Gk = GS + k * nck;
        for (int j = lane; j < nf; j += 32) {
            // channels + voltage pre-update (eden/Eden.cpp:5013-6107)
            const int ti = NT[j];
            const float v = XR[ti].x;
            VO[j] = v;
            float Iin, Gin, Isyn, Gsyn;
            block_currents(Gk, NB0[j], NB1[j], BKK, BKE, BKC, 0, v, Iin, Gin, Isyn, Gsyn);
            // (a model with gap junctions runs one-step windows: vsrc holds
            // every target's potential at this step's start)
            if (EDEN_KIND_GAP) Isyn += gap_current(m, t0 + ti, v, vsrc, init);
            const float A = NA[j];
            float Ich = 0.f, Gch = 0.f;
#ifdef EDEN_RTC_CHANNELS
            // the routine generated for this compartment's channel set
            if (!rtc_channels(NSIG[j], GT + CHQ[NCH0[j]], CHG, CHE, NCH0[j], v, A, Ich, Gch))
#endif
            for (int c = NCH0[j]; c < NCH1[j]; c++) {
                const int gi_pack = CHI[c];
                const float *q = GT + CHQ[c];
                float fopen = 1.0f;
                for (int gi = 0; gi < (gi_pack & 7); gi++) {
                    const float qo = q[gi];
                    const int inst = (gi_pack >> (3 + 5 * gi)) & 31;
                    for (int rr = 0; rr < inst; rr++) fopen = fopen * qo;
                }
                const float gs = CHG[c] * fopen;
                Ich += (gs * (CHE[c] - v) * 1e-5f) * A;
                Gch += (gs * 1e-5f) * A;
            }
            const float I = Ich + Iin + Isyn;
            const float G = Gch + Gin + Gsyn;
            const float C = NC[j];
            UP[ti].y = 1.0f * (G / C) + NIR[j];
            XR[ti].x = init ? v : v + (dt * (I + (v * G))) / C;
        }
        __syncwarp();
        if (!init) {
            if (f64) hines_window_f64(dt, XR, KL, UP, m.c_l + t0, LV, nlev, XD, PVD, RTD);
            else hines_window(dt, XR, KL, UP, LV, nlev);
        }
        // gate updates from this step's starting V and gate values (the
        // currents above used the values before the update, as the reference does)
        for (int q = lane; q < ngt; q += 32)
            GT[q] = gate_next_p(GP + q * kGateWords, m.gate_ext, init, dt, VO[GI_S[q]],
                                EDEN_KIND_GATEFORMS ? XR[NT[GI_S[q]]].x : 0.0f, GT[q]);
        // threshold crossings of the unit's spike sources (eden/Eden.cpp:6247-6252)
        for (int q0 = 0; q0 < ns; q0 += 32) {
            const int q = q0 + lane;
            bool spk = false;
            int src = -1;
            double tc = 0.0;
            if (q < ns) {
                const int sl = ST[q];
                src = SSRC[q];
                const float vo = VO[sl], vn = XR[NT[sl]].x;
                spk = vo < STHR[q] && STHR[q] < vn;
                if (spk) tc = crossing_time(tstep, dt, vo, vn, STHR[q]);
            }
            push_spike(m, spk, src, (int32_t)(step + 1), w.wpar, tc);
        }
        __syncwarp();
        if (!init) tstep += (double)dt;
    }
    // ---- write the unit back into the buffer that holds the window's final state
    float *vdst = m.v[w.par ^ (w.K & 1)];
    for (int i = lane; i < n; i += 32) vdst[t0 + i] = XR[i].x;
    for (int i = lane; i < ngt; i += 32) m.gate[gt0 + i] = GT[i];
}

// A batch of up to 32 point neurons over the window (izhikevich2007Cell,
// iaf*Cell, adExIaFCell; point_update), one lane each.
__device__ __forceinline__ void izh_window(const DevModel &m, const WindowArgs &w, const float *tk, int u, float *S) {
    const int lane = threadIdx.x & 31;
    const int t0 = m.un_t0[u], n = m.un_t1[u] - t0;
    const int r0 = m.un_r0[u], r1 = m.un_r1[u];
    // slice: V (two buffers), the parameters (stride n), then u, s and the kind
    float *P = S + 2 * n;
    float *SU = P + EDEN_POINT_PARAMS * n, *SS = SU + n;
    int32_t *KIND = (int32_t *)(SS + n);
    const int izh0 = m.t_izh[t0];
    for (int i = lane; i < n; i += 32) {
        const int iz = izh0 + i;
        stage_word(&S[w.par * n + i], &m.v[w.par][t0 + i]);
        for (int f = 0; f < EDEN_POINT_PARAMS; f++) stage_word(&P[f * n + i], &m.iz_p[(size_t)f * m.n_izh + iz]);
        stage_word(&SU[i], &m.iz_u[iz]);
        stage_word(&SS[i], &m.iz_s[iz]);
        stage_word(&KIND[i], &m.iz_kind[iz]);
    }
    stage_wait();
    __syncwarp();
    int par = w.par;
    const float dt = m.dt;
    for (int k = 0; k < w.K; k++) {
        const int64_t step = w.step0 + k;
        const bool init = step <= 0;
        const float *vin = S + par * n;
        float *vout = S + (par ^ 1) * n;
        const float *Gpk = m.Gp + (size_t)k * m.n_chunk;
        const int i = lane;
        bool spike = false;
        int src = -1;
        if (i < n) {
            const int t = t0 + i;
            const float v = vin[i];
            float Iin, Gin, Isyn, Gsyn;
            block_currents(Gpk, m.t_blk0[t], m.t_blk0[t + 1], m.bk_kind, m.bk_erev, m.bk_c0, 0, v, Iin, Gin, Isyn,
                           Gsyn);
            float uu = SU[i], ss = SS[i], vn;
            spike = point_update(KIND[i], P + i, n, init, tk[k], dt, v, Isyn + Iin, uu, ss, vn);
            vout[i] = vn;
            SU[i] = uu;
            SS[i] = ss;
            src = m.t_src[t];
        }
        push_spike(m, spike && src >= 0, src, (int32_t)(step + 1), w.wpar, no_time());
        if (!init && r1 > r0) {
            const int64_t row = (step - 1) % m.trace_cap;
            for (int q = r0 + lane; q < r1; q += 32) m.trace_buf[row * m.n_trace + m.gr_col[q]] = vin[m.gr_t[q]];
        }
        __syncwarp();
        par ^= 1;
    }
    for (int i = lane; i < n; i += 32) {
        m.v[par][t0 + i] = S[par * n + i];
        m.iz_u[izh0 + i] = SU[i];
        m.iz_s[izh0 + i] = SS[i];
    }
}

// This launch runs CTAs [cta_begin, cta_end), each a few units, one per warp.
// A block runs several CTAs in turn when there are more CTAs than blocks;
// their units are laid out differently in shared memory, so every warp of
// the block finishes its unit before any starts on the next CTA.
__global__ void __launch_bounds__(kCellThreads, 8) k_cells_t(DevModel m, const WindowArgs *tab, const WindowTimes *ttab,
                                                          const int *base, int idx, int cta_begin, int cta_end) {
    extern __shared__ __align__(16) float sm[];
    const WindowArgs w = tab[*base + idx];
    const float *tk = ttab[*base + idx].tk;
    const int warp = threadIdx.x >> 5;
    for (int cta = cta_begin + blockIdx.x; cta < cta_end; cta += gridDim.x) {
        const int u = m.cta_u0[cta] + warp;
        if (u < m.cta_u0[cta + 1]) {
            if (m.un_f[u] >= 0) { if (EDEN_KIND_FOREST) forest_window(m, w, u, sm + m.un_off[u]); }
            else if (EDEN_KIND_IZH) izh_window(m, w, tk, u, sm + m.un_off[u]);
        }
        if (cta + (int)gridDim.x < cta_end) __syncthreads();
    }
}

__global__ void k_bump(int *base, int by) { *base += by; }

}  // namespace eden
