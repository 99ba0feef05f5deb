// Library plumbing: error state, device arena, small shared kernels.
#include <stdarg.h>
#include <string.h>

#include "kdtree.cuh"

namespace rsg {

static thread_local Error g_err = {0, ""};

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

__global__ void k_slot_set(const int32_t *act, int32_t nact, int32_t *slot) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nact) slot[act[k]] = k;
}

__global__ void k_root_owner(const int32_t *rstart, const int32_t *rn, int32_t ntrees, int leaf,
                             int32_t *owner, int32_t *box_owner) {
    int t = blockIdx.x;
    if (t >= ntrees) return;
    int s = rstart[t], n = rn[t];
    int o = n > leaf ? t : -1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        box_owner[s + i] = t;
        owner[s + i] = o;
    }
}

}  // namespace rsg

extern "C" {

int rsg_version(void) { return 1; }

const char *rsg_last_error(void) { return rsg::g_err.msg; }

}  // extern "C"
