// prof.cu -- optional per-kernel timing with CUDA events (off by default).
//
// When enabled, every launch site of the library brackets its kernel with a
// pair of events on the launching stream; gcfg_profile_read() sums the
// device durations per kernel kind.  Used by bench.py to report the
// roofline of the dominant kernel from live measurements.
#include <mutex>
#include <vector>

#include "gcfg_internal.cuh"

namespace gcfg {

namespace {
struct Rec {
    int kind;
    cudaEvent_t a, b;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_free;
cudaEvent_t g_pending = nullptr;

cudaEvent_t get_event() {
    if (!g_free.empty()) {
        cudaEvent_t e = g_free.back();
        g_free.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

bool prof_on() { return g_on; }

void prof_begin(cudaStream_t st) {
    if (!g_on) return;
    std::lock_guard<std::mutex> lk(g_mu);
    g_pending = get_event();
    cudaEventRecord(g_pending, st);
}

void prof_end(int kind, cudaStream_t st) {
    if (!g_on) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_pending) return;
    cudaEvent_t b = get_event();
    cudaEventRecord(b, st);
    g_recs.push_back(Rec{kind, g_pending, b});
    g_pending = nullptr;
}

}  // namespace gcfg

using namespace gcfg;

extern "C" {

gcfg_status gcfg_profile_enable(int on) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on = on != 0;
    return GCFG_OK;
}

gcfg_status gcfg_profile_read(gcfg_prof_entry *out, int max_entries, int *n_out) {
    if (!out || max_entries < PK_COUNT_KINDS || !n_out) return GCFG_ERR_INVALID;
    std::lock_guard<std::mutex> lk(g_mu);
    for (int k = 0; k < PK_COUNT_KINDS; ++k) {
        out[k].kind = k;
        out[k].launches = 0;
        out[k].ms = 0.0;
    }
    for (auto &r : g_recs) {
        if (cudaEventSynchronize(r.b) != cudaSuccess) return GCFG_ERR_CUDA;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        out[r.kind].launches++;
        out[r.kind].ms += ms;
        g_free.push_back(r.a);
        g_free.push_back(r.b);
    }
    g_recs.clear();
    *n_out = PK_COUNT_KINDS;
    return GCFG_OK;
}

}  // extern "C"
