// Library plumbing: error state, device arena, small shared kernels.
#include <stdarg.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "kdtree.cuh"

namespace rsg {

static thread_local Error g_err = {0, ""};
static thread_local int64_t g_stats[RSG_STAT_COUNT];

int64_t *last_stats() { return g_stats; }

static Tuning g_tuning;
Tuning &tuning() { return g_tuning; }

void set_error(int code, const char *fmt, ...) {
    g_err.code = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err.msg, sizeof(g_err.msg), fmt, ap);
    va_end(ap);
}

int error_code() { return g_err.code ? g_err.code : RSG_ERR_CUDA; }

void Arena::reserve(size_t bytes) {
    if (bytes <= cap) return;
    if (base) cudaFree(base);
    base = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 8 + (64u << 20);
    cudaError_t e = cudaMalloc(&base, want);
    if (e != cudaSuccess) {
        base = nullptr;
        set_error(RSG_ERR_CUDA, "arena cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
        throw Failure();
    }
    cap = want;
}

void *Arena::take(size_t bytes) {
    size_t off = (used + 255) & ~(size_t)255;
    if (off + bytes > cap) {
        set_error(RSG_ERR_LIMIT, "device arena exhausted (%zu + %zu > %zu)", off, bytes, cap);
        throw Failure();
    }
    used = off + bytes;
    if (used > peak) peak = used;
    return base + off;
}

Arena::~Arena() {
    if (base) cudaFree(base);
}

__global__ void k_slot_set(const int32_t *act, const LevelState *ls, int32_t *slot) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ls->nact) slot[act[k]] = k;
}
__global__ void k_iota_i32(int32_t *a, int32_t n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) a[k] = k;
}
// After k_children: the level's new nodes become [base, base + nnew), and
// those that split again are the next level's active nodes.
__global__ void k_level_advance(LevelState *ls, const int64_t *off, int32_t *lvl_end,
                                int32_t level) {
    if (threadIdx.x || blockIdx.x) return;
    const int64_t t = off[ls->nact];
    ls->base = ls->nnodes;
    ls->nnew = ls->err ? 0 : 2 * (int32_t)(t >> 32);
    ls->nnodes += ls->nnew;
    ls->nact = ls->err ? 0 : (int32_t)(t & 0xffffffffu);
    lvl_end[level] = ls->nnodes;
}

__global__ void k_root_owner(const int32_t *rstart, const int32_t *rn, int32_t ntrees, int leaf,
                             int32_t *owner, int32_t *box_owner) {
    int t = blockIdx.x;  // tree; blockIdx.y strides through its elements
    if (t >= ntrees) return;
    int s = rstart[t], n = rn[t];
    int o = n > leaf ? t : -1;
    for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < n; i += gridDim.y * blockDim.x) {
        box_owner[s + i] = t;
        owner[s + i] = o;
    }
}

// ---- phase timers ----------------------------------------------------------
#include <chrono>
#include <map>
static int g_timing = -1;
static std::map<std::string, double> g_phase;
static std::chrono::steady_clock::time_point g_last;
static std::vector<std::string> g_phase_order;
void phase_mark(cudaStream_t st, const char *name) {
    if (g_timing < 0) g_timing = getenv("RSG_TIMING") ? 1 : 0;
    if (!g_timing) return;
    cudaStreamSynchronize(st);
    auto now = std::chrono::steady_clock::now();
    if (name && *name) {
        if (!g_phase.count(name)) g_phase_order.push_back(name);
        g_phase[name] += std::chrono::duration<double, std::milli>(now - g_last).count();
    }
    g_last = now;
}
void phase_report() {
    if (g_timing <= 0) return;
    for (auto &k : g_phase_order) fprintf(stderr, "  [phase] %-28s %10.2f ms\n", k.c_str(), g_phase[k]);
    g_phase.clear();
    g_phase_order.clear();
}

// ---- launch accounting and event timing of one selected kernel -----------
static LaunchStats g_ls;
static std::string g_prof_name;
static std::unordered_map<const void *, bool> g_prof_cache;
struct ProfRec {
    cudaEvent_t a, b;
    const void *func;
};
static std::vector<ProfRec> g_prof_ev;
static std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_prof_pool;
static size_t g_prof_used = 0;

LaunchStats &launch_stats() { return g_ls; }

bool prof_match(const void *func) {
    auto it = g_prof_cache.find(func);
    if (it != g_prof_cache.end()) return it->second;
    const char *nm = nullptr;
    bool m = false;
    if (g_prof_name == "*") m = true;  // every kernel
    else if (cudaFuncGetName(&nm, func) == cudaSuccess && nm)
        m = strstr(nm, g_prof_name.c_str()) != nullptr;
    g_prof_cache[func] = m;
    return m;
}
void prof_begin(cudaStream_t st, const void *func) {
    if (g_prof_used == g_prof_pool.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        g_prof_pool.push_back({a, b});
    }
    auto &e = g_prof_pool[g_prof_used++];
    g_prof_ev.push_back({e.first, e.second, func});
    cudaEventRecord(g_prof_ev.back().a, st);
}
void prof_end(cudaStream_t st) { cudaEventRecord(g_prof_ev.back().b, st); }

}  // namespace rsg

extern "C" {

int64_t rsg_launch_count(void) { return rsg::g_ls.launches; }

int rsg_profile_select(const char *kernel_substring) {
    rsg::g_prof_name = kernel_substring ? kernel_substring : "";
    rsg::g_prof_cache.clear();
    rsg::g_prof_ev.clear();
    rsg::g_prof_used = 0;
    rsg::g_ls.selecting = !rsg::g_prof_name.empty();
    return 0;
}

int rsg_profile_read(int64_t *launches, double *total_ms) {
    double t = 0;
    for (auto &e : rsg::g_prof_ev) {
        float ms = 0;
        if (cudaEventSynchronize(e.b) != cudaSuccess) return RSG_ERR_CUDA;
        cudaEventElapsedTime(&ms, e.a, e.b);
        t += ms;
    }
    *launches = (int64_t)rsg::g_prof_ev.size();
    *total_ms = t;
    rsg::g_prof_ev.clear();
    rsg::g_prof_used = 0;
    return 0;
}

int64_t rsg_profile_table(char *buf, int64_t cap) {
    struct Agg {
        int64_t n = 0;
        double ms = 0, gap = 0;
    };
    std::unordered_map<std::string, Agg> agg;
    const rsg::ProfRec *prev = nullptr;
    for (auto &e : rsg::g_prof_ev) {
        float ms = 0, gap = 0;
        if (cudaEventSynchronize(e.b) != cudaSuccess) return RSG_ERR_CUDA;
        cudaEventElapsedTime(&ms, e.a, e.b);
        // time since the previous timed launch ended: work that is not timed
        // (library scans and sorts, copies) and the host's round trips
        if (prev) cudaEventElapsedTime(&gap, prev->b, e.a);
        prev = &e;
        const char *nm = nullptr;
        std::string name = (cudaFuncGetName(&nm, e.func) == cudaSuccess && nm) ? nm : "?";
        auto &r = agg[name];
        r.n++;
        r.ms += ms;
        r.gap += gap > 0 ? gap : 0;
    }
    std::vector<std::pair<double, std::string>> rows;
    for (auto &kv : agg) {
        char line[1024];
        snprintf(line, sizeof(line), "%s\t%lld\t%.6f\t%.6f\n", kv.first.c_str(),
                 (long long)kv.second.n, kv.second.ms, kv.second.gap);
        rows.push_back({kv.second.ms, line});
    }
    std::sort(rows.begin(), rows.end(), [](const auto &x, const auto &y) { return x.first > y.first; });
    std::string out;
    for (auto &r : rows) out += r.second;
    rsg::g_prof_ev.clear();
    rsg::g_prof_used = 0;
    if (buf && cap > 0) {
        size_t n = out.size() < (size_t)cap - 1 ? out.size() : (size_t)cap - 1;
        memcpy(buf, out.data(), n);
        buf[n] = 0;
    }
    return (int64_t)out.size();
}

int rsg_last_stats(int64_t *vals, int32_t n) {
    if (!vals || n < 0) return RSG_ERR_ARGS;
    for (int32_t i = 0; i < n && i < RSG_STAT_COUNT; i++) vals[i] = rsg::g_stats[i];
    return RSG_OK;
}

int rsg_version(void) { return 1; }

const char *rsg_last_error(void) { return rsg::g_err.msg; }

}  // extern "C"
