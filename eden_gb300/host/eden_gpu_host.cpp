// eden_gpu_host: a C++ host that runs a lowered network on the GPU through
// the C ABI of libeden_gpu (include/eden_gpu.h) and writes the reference's
// output files.
//
// It plays the part the step loop of eden/Eden.cpp:11488-11938 plays in the
// reference: the four initialisation passes, then the simulation steps in
// chunks between logger flushes, each chunk one edenGpuRun call followed by
// one edenGpuFetchRecords, the records written as the reference's
// OutputFile (one line per sample: the time in seconds, then each column in
// its output units, "%+16.8g", eden/Eden.cpp:10856-10871) and
// EventOutputFile in TIME_ID form (one line per event, time then the
// selection id, 10914-10922) with its Config / Setup / Run timing line
// (11951).  The network comes from a file written by eden_gb300/model_file.py
// (every EdenGpuModel field by name, then the run's recorded targets, their
// output scales, the event columns and the step count); a host that parses
// NeuroML itself fills the same struct from its own model instead.
//
//   eden_gpu_host MODEL_FILE TRAJECTORY_FILE EVENT_FILE [plain|batched] [chunk_steps]
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "eden_gpu.h"

namespace {

struct Field {
    int type = -1;      // 0 int32, 1 int64, 2 float32, 3 float64, 4 bytes
    uint64_t count = 0;
    std::vector<uint64_t> data;  // 8-byte aligned storage
    const void *ptr() const { return data.data(); }
};

bool read_model_file(const char *path, std::map<std::string, Field> &out, std::string &err) {
    FILE *f = fopen(path, "rb");
    if (!f) { err = std::string("cannot open ") + path; return false; }
    char magic[8];
    if (fread(magic, 1, 8, f) != 8 || memcmp(magic, "EDENGPU1", 8) != 0) {
        err = "not a lowered-model file (bad magic)";
        fclose(f);
        return false;
    }
    static const size_t kSize[5] = {4, 8, 4, 8, 1};
    while (true) {
        uint16_t nlen;
        if (fread(&nlen, 2, 1, f) != 1) break;
        std::string name(nlen, '\0');
        uint8_t type;
        uint64_t count;
        if (fread(&name[0], 1, nlen, f) != nlen || fread(&type, 1, 1, f) != 1 || fread(&count, 8, 1, f) != 1 ||
            type > 4) {
            err = "truncated record header";
            fclose(f);
            return false;
        }
        Field fl;
        fl.type = type;
        fl.count = count;
        const size_t bytes = kSize[type] * count;
        fl.data.assign(bytes / 8 + 1, 0);
        if (fread(fl.data.data(), 1, bytes, f) != bytes) {
            err = "truncated record " + name;
            fclose(f);
            return false;
        }
        out[name] = std::move(fl);
    }
    fclose(f);
    return true;
}

// Typed views of the records; a missing pointer field is NULL, a missing
// count is 0.
struct Reader {
    const std::map<std::string, Field> &rec;
    const Field *get(const char *name) const {
        auto it = rec.find(name);
        return it == rec.end() ? nullptr : &it->second;
    }
    int64_t integer(const char *name) const {
        const Field *f = get(name);
        if (!f || f->count == 0) return 0;
        return f->type == 1 ? *(const int64_t *)f->ptr() : *(const int32_t *)f->ptr();
    }
    float real(const char *name) const {
        const Field *f = get(name);
        return f && f->count ? *(const float *)f->ptr() : 0.0f;
    }
    template <typename T> const T *array(const char *name) const {
        const Field *f = get(name);
        return f ? (const T *)f->ptr() : nullptr;
    }
};

void fill_model(const Reader &r, EdenGpuModel &m) {
    memset(&m, 0, sizeof(m));
    m.abi_version = (int32_t)r.integer("abi_version");
    m.dt = r.real("dt");
    m.seed = r.integer("seed");
#define I32(f) m.f = (int32_t)r.integer(#f)
#define I64(f) m.f = r.integer(#f)
#define PTR(f, T) m.f = r.array<T>(#f)
    I32(n_phys); PTR(phys_comp_off, int32_t);
    I32(n_comp); PTR(comp_parent, int32_t); PTR(comp_c, float); PTR(comp_r_axial, float);
    PTR(comp_area, float); PTR(comp_inv_rc, float); PTR(comp_v0, float);
    I32(n_chan_types); PTR(chan_types, EdenGpuChannelType);
    PTR(comp_chan_off, int32_t); PTR(chan_type, int32_t); PTR(chan_gbase, float); PTR(chan_erev, float);
    I32(n_izh); PTR(izh_params, float);
    I32(n_src); PTR(src_target, int32_t); PTR(src_threshold, float); PTR(src_cell_seed, int32_t);
    I32(n_syn_types); PTR(syn_types, EdenGpuSynapseType);
    I64(n_syn); PTR(syn_target, int32_t); PTR(syn_type, int32_t); PTR(syn_src, int32_t);
    PTR(syn_weight, float); PTR(syn_delay, float);
    I64(n_pois); PTR(pois_target, int32_t); PTR(pois_type, int32_t); PTR(pois_rate, float);
    PTR(pois_weight, float); PTR(pois_src, int32_t); PTR(pois_instance, int32_t);
    I64(n_pulse); PTR(pulse_target, int32_t); PTR(pulse_start, float); PTR(pulse_duration, float);
    PTR(pulse_amplitude, float); PTR(pulse_weight, float);
    I64(n_ext); PTR(ext_src, int32_t); PTR(ext_step, int64_t);
    PTR(izh_kind, int32_t);
    I64(n_timed); PTR(timed_target, int32_t); PTR(timed_type, int32_t); PTR(timed_weight, float);
    PTR(timed_off, int64_t); PTR(timed_step, int64_t);
    I64(n_wave); PTR(wave_target, int32_t); PTR(wave_shape, int32_t); PTR(wave_params, float);
    PTR(wave_weight, float);
    PTR(pois_rng_base, int32_t);
    I64(n_clamp); PTR(clamp_target, int32_t); PTR(clamp_params, float); PTR(clamp_weight, float);
    I64(n_gap); PTR(gap_target, int32_t); PTR(gap_peer, int32_t); PTR(gap_conductance, float);
    PTR(gap_weight, float);
    I32(cable_solver);
    I64(n_graded); PTR(graded_target, int32_t); PTR(graded_peer, int32_t); PTR(graded_params, float);
    PTR(graded_weight, float);
#undef I32
#undef I64
#undef PTR
}

double seconds_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s MODEL_FILE TRAJECTORY_FILE EVENT_FILE [plain|batched] [chunk_steps]\n", argv[0]);
        return 2;
    }
    const auto t_config = std::chrono::steady_clock::now();
    std::map<std::string, Field> rec;
    std::string err;
    if (!read_model_file(argv[1], rec, err)) {
        fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    const Reader r{rec};
    EdenGpuModel model;
    fill_model(r, model);
    if (model.abi_version != edenGpuAbiVersion()) {
        fprintf(stderr, "model file is for ABI version %d, the library is %d\n", model.abi_version,
                edenGpuAbiVersion());
        return 1;
    }
    const Field *tt = r.get("run.trace_target");
    const Field *sc = r.get("run.trace_scale");
    const Field *es = r.get("run.event_src");
    const Field *ei = r.get("run.event_id");
    const int64_t n_steps = r.integer("run.n_steps");
    int mode = (int)r.integer("run.mode");
    if (argc > 4) mode = strcmp(argv[4], "plain") == 0 ? EDEN_MODE_PLAIN : EDEN_MODE_BATCHED;
    const int chunk = argc > 5 ? std::max(1, atoi(argv[5])) : 4096;
    const int n_trace = tt ? (int)tt->count : 0;
    const double *scale = sc ? (const double *)sc->ptr() : nullptr;
    // event columns: selection ids, and the columns of each spike source
    std::vector<std::string> ids;
    if (ei) {
        const char *p = (const char *)ei->ptr();
        std::string cur;
        for (uint64_t k = 0; k < ei->count; k++) {
            if (p[k] == '\n') { ids.push_back(cur); cur.clear(); }
            else cur += p[k];
        }
        ids.push_back(cur);
    }
    std::vector<std::vector<int>> cols_of_src(model.n_src);
    if (es)
        for (uint64_t j = 0; j < es->count; j++) {
            const int s = ((const int32_t *)es->ptr())[j];
            if (s >= 0 && s < model.n_src) cols_of_src[s].push_back((int)j);
        }
    const double config_s = seconds_since(t_config);

    const auto t_setup = std::chrono::steady_clock::now();
    EdenGpuOptions opt;
    memset(&opt, 0, sizeof(opt));
    opt.mode = mode;
    opt.record_capacity_steps = chunk;
    opt.spike_capacity = 1 << 22;
    opt.n_trace = n_trace;
    opt.trace_target = tt ? (const int32_t *)tt->ptr() : nullptr;
    EdenGpuCtx *ctx = nullptr;
    if (edenGpuCreate(&model, &opt, &ctx) != EDEN_GPU_OK) {
        fprintf(stderr, "GPU set-up failed: %s\n", ctx ? edenGpuLastError(ctx) : "no context");
        edenGpuDestroy(ctx);
        return 1;
    }
    const double setup_s = seconds_since(t_setup);

    FILE *ftraj = fopen(argv[2], "w"), *fev = fopen(argv[3], "w");
    if (!ftraj || !fev) {
        fprintf(stderr, "cannot open the output files\n");
        edenGpuDestroy(ctx);
        return 1;
    }
    const auto t_run = std::chrono::steady_clock::now();
    // simulation time of each step, accumulated in double from the float dt
    // as the reference's loop does (eden/Eden.cpp:11486, 11931): steps <= 1
    // run at 0, step k at the sum of k - 1 dts
    std::vector<double> t_us(n_steps + 2, 0.0);
    for (int64_t k = 2; k < (int64_t)t_us.size(); k++) t_us[k] = t_us[k - 1] + (double)model.dt;
    std::vector<float> trace((size_t)chunk * std::max(n_trace, 1));
    std::vector<int64_t> trace_step(chunk), spike_step(opt.spike_capacity);
    std::vector<int32_t> spike_src(opt.spike_capacity);
    int rc = edenGpuRun(ctx, -3, 4);  // the four initialisation passes
    int64_t step = 1;
    std::vector<std::pair<int, int64_t>> events;  // (column, step) of the chunk's events
    while (rc == EDEN_GPU_OK && step <= n_steps) {
        const int64_t k = std::min<int64_t>(chunk, n_steps - step + 1);
        rc = edenGpuRun(ctx, step, k);
        if (rc != EDEN_GPU_OK) break;
        EdenGpuRecords out = {trace.data(), trace_step.data(), (int64_t)chunk,
                              spike_src.data(), spike_step.data(), (int64_t)opt.spike_capacity, 0, 0};
        rc = edenGpuFetchRecords(ctx, &out);
        if (rc != EDEN_GPU_OK) break;
        for (int64_t i = 0; i < out.n_trace_samples; i++) {
            fprintf(ftraj, "%+16.8g", t_us[trace_step[i]] * 1e-6);
            for (int j = 0; j < n_trace; j++)
                fprintf(ftraj, " %+16.8g", (double)trace[i * n_trace + j] * (scale ? scale[j] : 1.0));
            fputc('\n', ftraj);
        }
        // one frame per logging step with events, columns in selection order
        events.clear();
        for (int64_t i = 0; i < out.n_spikes; i++)
            if (spike_src[i] >= 0 && spike_src[i] < model.n_src && spike_step[i] <= n_steps)
                for (int c : cols_of_src[spike_src[i]]) events.push_back({c, spike_step[i]});
        std::sort(events.begin(), events.end(), [](const auto &a, const auto &b) {
            return a.second != b.second ? a.second < b.second : a.first < b.first;
        });
        for (const auto &e : events)
            fprintf(fev, "%+16.8g %s\n", t_us[e.second] * 1e-6, e.first < (int)ids.size() ? ids[e.first].c_str() : "?");
        step += k;
    }
    const double run_s = seconds_since(t_run);
    fclose(ftraj);
    fclose(fev);
    if (rc != EDEN_GPU_OK) {
        fprintf(stderr, "run failed: %s\n", edenGpuLastError(ctx));
        edenGpuDestroy(ctx);
        return 1;
    }
    printf("Config: %g Setup: %g Run: %g \n", config_s, setup_s, run_s);
    edenGpuDestroy(ctx);
    return 0;
}
