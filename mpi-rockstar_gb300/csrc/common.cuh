// Shared definitions for the GB300 halo-finding kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "launch.cuh"
#include "rockstar_gb300.h"

namespace rsg {

// Error plumbing: every CUDA call is checked on the host; failures are
// recorded in a thread-local status that the C-ABI returns to the caller.
struct Error {
    int code;
    char msg[256];
};
void set_error(int code, const char *fmt, ...);
int error_code();
#define RSG_CUDA(call)                                                                 \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ::rsg::set_error(RSG_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,  \
                             cudaGetErrorString(e_));                                  \
            throw ::rsg::Failure();                                                    \
        }                                                                              \
    } while (0)
#define RSG_CHECK_LAUNCH() RSG_CUDA(cudaGetLastError())
struct Failure {};

// Working record for every tree build over particles: positions first so the
// record can be loaded as two float4; `ridx` points back at the caller's
// particle (the role the hijacked id plays in src/groupies.c:684-686).
struct __align__(16) Rec {
    float pos[6];
    int32_t ridx;
    int32_t aux;
};
static_assert(sizeof(Rec) == 32, "Rec must be 32 bytes");

// Node of a median-of-extent kd-tree (layout of src/fast3tree.c:184-193,
// indices instead of pointers).
template <int D>
struct KNode {
    float mn[D], mx[D];
    int32_t start, n;
    int32_t div;     // split dimension, -1 for a leaf
    int32_t left;    // right child is left + 1
    int32_t parent;
    int32_t tree;    // index of the tree (forest builds)
};

// Device-side scratch arena: one cudaMalloc, bump allocation per call.
struct Arena {
    char *base = nullptr;
    size_t cap = 0, used = 0, peak = 0;
    bool fixed = false;  // borrowed storage: nothing beside it may be allocated
    void reserve(size_t bytes);
    void *take(size_t bytes);
    template <class T>
    T *get(size_t n) { return (T *)take(n * sizeof(T)); }
    void reset() { used = 0; }
    ~Arena();
};

// Exact IEEE float arithmetic without FMA contraction: the reference
// evaluates `dist += dx*dx` as a rounded multiply followed by a rounded add.
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
// The reference's (float)sqrt((double)x) for a float x.  Rounding the exact
// square root to double and then to float gives the float rounding of the
// exact root, because 53 >= 2 * 24 + 2 makes double rounding innocuous for
// square roots (Figueroa, "When is double rounding innocuous?", 1995), so
// the IEEE float square root is bit-identical and keeps the FP64 pipe free.
__device__ __forceinline__ float sqrt_fd(float x) { return __fsqrt_rn(x); }
// hi + lo += y with Knuth's two-sum: hi takes the rounded sum, lo gathers the
// exact rounding errors (explicit round-to-nearest operations, so nothing is
// contracted or reordered).
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float y) {
    float s = __fadd_rn(hi, y);
    float bp = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(y, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// Order-preserving float <-> uint mapping for atomic min/max on floats.
__device__ __forceinline__ unsigned f2ord(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

inline int nblk(int64_t n, int t) { return (int)((n + t - 1) / t); }

// Phase timer: with RSG_TIMING set in the environment, synchronises the
// stream at each mark and accumulates wall time per phase name; the totals
// are printed to stderr by phase_report().
void phase_mark(cudaStream_t st, const char *name);
void phase_report();

// Counters of the last call on the calling thread (rsg_last_stats); the
// indices are the RSG_STAT_* constants of the public header.
int64_t *last_stats();

// Size-class thresholds and chunk sizes of the batched form; process-wide,
// set through rsg_set_tuning.  They change speed only: choices stay exact
// and sums change at most by FP64 rounding.
struct Tuning {
    int32_t asc_bucket_min = 64;  // nodes with more halos scan Morton buckets
    int32_t bh_huge = 65536;      // Barnes-Hut nodes above: chunked pass
    int32_t bh_chunk = 16384;     // points per chunk of that pass
    int32_t seg_max = 8192;       // records per potential-set copy segment
    int32_t norm_chunk = 4096;    // records per chunk of the chunked norm_sd
    int32_t bp_big = 16384;       // halos above: chunked basic properties
    int32_t bp_chunk = 4096;      // particles per chunk of those
};
Tuning &tuning();

#define RSG_STACK 96
#define RSG_STACK6 128

// Blackwell's packed FP32 arithmetic: two floats per 64-bit register (the
// lower-addressed value in the low half), each lane rounded as the scalar
// operation (.rn), so a packed subtraction or square gives the same floats
// as two scalar ones.
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_sqr(unsigned long long a) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(r) : "l"(a));
    return r;
}
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_split(unsigned long long v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

}  // namespace rsg
