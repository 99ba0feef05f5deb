// Exact GPU version of partition_sort_particles (src/fof.c:184-224): each
// segment is split at the midpoint of its label range with the same
// two-pointer swap that the kd-tree build uses (closed form in kdtree.cuh),
// then both halves recurse.  Runs level-synchronously over many segments.
#pragma once
#include "kdtree.cuh"

namespace rsg {

struct LSeg {
    int32_t *start, *n;   // active segments
    int32_t *mn, *mx;     // label range
    int32_t *pivot, *m, *q;
};

// owner[i]: the active segment holding element i (segments are disjoint and
// listed by ascending start), -1 outside every segment.
static __global__ void k_ls_owner(const int32_t *start, const int32_t *n, int32_t ns, int64_t M,
                                  int32_t *owner) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int lo = 0, hi = ns - 1, k = -1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        if (start[mid] <= i) {
            k = mid;
            lo = mid + 1;
        } else {
            hi = mid - 1;
        }
    }
    owner[i] = (k >= 0 && i < (int64_t)start[k] + n[k]) ? k : -1;
}
static __global__ void k_ls_init(LSeg S, int32_t ns) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    S.mn[k] = 0x7fffffff;
    S.mx[k] = (int32_t)0x80000000;
}
// Label range of every segment.  A thread reads ITEMS consecutive elements;
// threads whose elements all belong to one segment combine their ranges
// with the other lanes of that segment before the atomics (a large segment
// gets one atomic pair per warp instead of one per thread).
template <int ITEMS>
static __global__ void k_ls_minmax(const int32_t *lab, int64_t M, const int32_t *owner, LSeg S) {
    const unsigned FULL = 0xffffffffu;
    int64_t i0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * ITEMS;
    int first = -2;  // owner shared by all of this thread's elements, -1 mixed/none
    int cur = -1, lo = 0x7fffffff, hi = (int)0x80000000;
    for (int it = 0; it < ITEMS; it++) {
        int64_t i = i0 + it;
        int a = (i < M) ? owner[i] : -1;
        if (first == -2) first = a;
        else if (a != first) first = -1;
        if (a != cur) {
            if (cur >= 0 && first == -1) {  // mixed: this run goes out on its own
                atomicMin(&S.mn[cur], lo);
                atomicMax(&S.mx[cur], hi);
            }
            cur = a;
            lo = 0x7fffffff;
            hi = (int)0x80000000;
        }
        if (a < 0) continue;
        int v = lab[i];
        lo = min(lo, v);
        hi = max(hi, v);
    }
    bool uni = first >= 0;  // every element in one segment: combine across the warp
    unsigned grp = __match_any_sync(FULL, uni ? first : -1);
    if (uni) {
        int glo = __reduce_min_sync(grp, lo), ghi = __reduce_max_sync(grp, hi);
        if ((threadIdx.x & 31) == __ffs(grp) - 1) {
            atomicMin(&S.mn[first], glo);
            atomicMax(&S.mx[first], ghi);
        }
    } else if (cur >= 0) {
        atomicMin(&S.mn[cur], lo);
        atomicMax(&S.mx[cur], hi);
    }
}
// pivot = min + (max - min) / 2 (src/fof.c:201); segments whose labels are
// all equal are finished (no element is "big").
static __global__ void k_ls_pivot(LSeg S, int32_t ns) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    int64_t lo = S.mn[k], hi = S.mx[k];
    S.pivot[k] = (lo == hi) ? 0x7fffffff : (int32_t)(lo + (hi - lo) / 2);
}
static __global__ void k_ls_flags(const int32_t *lab, int64_t M, const int32_t *owner, LSeg S,
                           int32_t *flag) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i > M) return;
    int f = 0;
    if (i < M) {
        int a = owner[i];
        if (a >= 0) f = lab[i] > S.pivot[a];
    }
    flag[i] = f;
}
static __global__ void k_ls_counts(LSeg S, int32_t ns, const int32_t *rank) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ns) return;
    int s = S.start[k], n = S.n[k];
    int B = rank[s + n] - rank[s];
    int m = n - B;
    S.m[k] = m;
    S.q[k] = rank[s + m] - rank[s];
}
static __global__ void k_ls_tables(int64_t M, const int32_t *owner, LSeg S, const int32_t *flag,
                            const int32_t *rank, int32_t *fb, int32_t *bs) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int a = owner[i];
    if (a < 0) return;
    int s = S.start[a];
    int l = (int)(i - s);
    int br = rank[i] - rank[s];
    int sr = l - br;
    int m = S.m[a];
    if (flag[i] && l < m) fb[s + br] = l;
    if (!flag[i] && l >= m) bs[s + (m - 1 - sr)] = l;
}
template <class T>
__global__ void k_ls_scatter(int64_t M, const int32_t *owner, LSeg S, const int32_t *flag,
                             const int32_t *rank, const int32_t *fb, const int32_t *bs,
                             const T *src, T *dst, const int32_t *lsrc, int32_t *ldst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int a = owner[i];
    if (a < 0) return;
    int s = S.start[a], n = S.n[a];
    int l = (int)(i - s);
    int br = rank[i] - rank[s];
    int sr = l - br;
    int m = S.m[a], q = S.q[a];
    int big = flag[i];
    int d;
    if (!big && l < m) d = l;
    else if (big && l < m) d = (br == 0) ? n - 1 : bs[s + br - 1] - 1;
    else if (!big) d = fb[s + (m - 1 - sr)];
    else {
        int pos_last = (q > 0) ? bs[s + q - 1] : n;
        if (l > pos_last) d = l - 1;
        else if (pos_last - m >= 2) d = (l == m) ? pos_last - 1 : l - 1;
        else d = l;
    }
    dst[s + d] = src[i];
    ldst[s + d] = lsrc[i];
}
// After a round: every element moves to the half of its segment it now
// lies in; a half that goes on (flag) gets its compacted index (nidx), and
// the elements of a half that is finished are final and are copied from the
// buffer the round wrote (src) to the output arrays when they differ.
template <class T>
__global__ void k_ls_owner_next(int64_t M, int32_t *owner, LSeg S, const int32_t *nflag,
                                const int32_t *nidx, const T *src, T *dst, const int32_t *lsrc,
                                int32_t *ldst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= M) return;
    int a = owner[i];
    if (a < 0) return;
    int h = 2 * a + ((i - S.start[a]) < S.m[a] ? 0 : 1);
    if (nflag[h]) {
        owner[i] = nidx[h];
        return;
    }
    owner[i] = -1;
    if (src != dst) {
        dst[i] = src[i];
        ldst[i] = lsrc[i];
    }
}
// next round: both halves of every split segment with >= 2 elements
static __global__ void k_ls_next(LSeg S, int32_t ns, int32_t *ns_start, int32_t *ns_n, int32_t *flag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == ns) flag[2 * ns] = 0;  // the scan's last entry
    if (k >= ns) return;
    int s = S.start[k], n = S.n[k], m = S.m[k];
    bool split = S.mn[k] != S.mx[k];
    ns_start[2 * k] = s;
    ns_n[2 * k] = m;
    ns_start[2 * k + 1] = s + m;
    ns_n[2 * k + 1] = n - m;
    flag[2 * k] = split && m >= 2;
    flag[2 * k + 1] = split && (n - m) >= 2;
}

// Sorts W (and its labels) inside every segment (host arrays hs/hn) the way
// the reference's recursive partition does.
template <class T>
void partition_sort_labels(Arena &ar, T *W, int32_t *lab, int64_t M,
                           const std::vector<int32_t> &hs, const std::vector<int32_t> &hn,
                           cudaStream_t st);

}  // namespace rsg

namespace rsg {

template <class T>
void partition_sort_labels(Arena &ar, T *W, int32_t *lab, int64_t M,
                           const std::vector<int32_t> &hs, const std::vector<int32_t> &hn,
                           cudaStream_t st) {
    std::vector<int32_t> s0, n0;
    for (size_t k = 0; k < hs.size(); k++)
        if (hn[k] >= 2) {
            s0.push_back(hs[k]);
            n0.push_back(hn[k]);
        }
    int32_t ns = (int32_t)s0.size();
    if (ns == 0) return;
    const int T_ = 256;
    size_t mark = ar.used;
    int64_t cap = (int64_t)ns > M / 2 + 1 ? ns : M / 2 + 1;
    LSeg S;
    S.start = ar.get<int32_t>(cap); S.n = ar.get<int32_t>(cap);
    S.mn = ar.get<int32_t>(cap); S.mx = ar.get<int32_t>(cap);
    S.pivot = ar.get<int32_t>(cap); S.m = ar.get<int32_t>(cap); S.q = ar.get<int32_t>(cap);
    int32_t *nst = ar.get<int32_t>(2 * cap), *nn = ar.get<int32_t>(2 * cap);
    int32_t *nflag = ar.get<int32_t>(2 * cap + 1), *nidx = ar.get<int32_t>(2 * cap + 1);
    int32_t *owner = ar.get<int32_t>(M), *flag = ar.get<int32_t>(M + 1), *rank = ar.get<int32_t>(M + 1);
    int32_t *fb = ar.get<int32_t>(M), *bs = ar.get<int32_t>(M);
    T *tw = ar.get<T>(M);
    int32_t *tl = ar.get<int32_t>(M);
    int *cnt = ar.get<int>(1);
    size_t b1 = 0, b2 = 0, b3 = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b1, flag, rank, (int)(M + 1), st);
    cub::DeviceSelect::Flagged(nullptr, b2, nst, nflag, S.start, cnt, (int)(2 * cap), st);
    cub::DeviceScan::ExclusiveSum(nullptr, b3, nflag, nidx, (int)(2 * cap + 1), st);
    if (b2 > b1) b1 = b2;
    if (b3 > b1) b1 = b3;
    void *tmp = ar.take(b1 + 256);
    size_t tb = b1 + 256;
    RSG_CUDA(cudaMemcpyAsync(S.start, s0.data(), 4 * ns, cudaMemcpyHostToDevice, st));
    RSG_CUDA(cudaMemcpyAsync(S.n, n0.data(), 4 * ns, cudaMemcpyHostToDevice, st));
    // rounds scatter back and forth between (W, lab) and (tw, tl); an
    // element is copied to (W, lab) once, when its segment is finished
    T *wb[2] = {W, tw};
    int32_t *lb[2] = {lab, tl};
    int cur = 0;
    launch(k_ls_owner, nblk(M, T_), T_, 0, st, (const int32_t *)S.start, (const int32_t *)S.n, ns,
           M, owner);
    for (int round = 0; ns > 0; round++) {
        if (round > 200) {
            set_error(RSG_ERR_LIMIT, "label partition sort did not terminate");
            throw Failure();
        }
        launch(k_ls_init, nblk(ns, T_), T_, 0, st, S, ns);
        launch(k_ls_minmax<8>, nblk((M + 7) / 8, T_), T_, 0, st, (const int32_t *)lb[cur], M,
               (const int32_t *)owner, S);
        launch(k_ls_pivot, nblk(ns, T_), T_, 0, st, S, ns);
        launch(k_ls_flags, nblk(M + 1, T_), T_, 0, st, (const int32_t *)lb[cur], M,
               (const int32_t *)owner, S, flag);
        cub::DeviceScan::ExclusiveSum(tmp, tb, flag, rank, (int)(M + 1), st);
        launch(k_ls_counts, nblk(ns, T_), T_, 0, st, S, ns, rank);
        launch(k_ls_tables, nblk(M, T_), T_, 0, st, M, owner, S, flag, rank, fb, bs);
        launch(k_ls_scatter<T>, nblk(M, T_), T_, 0, st, M, owner, S, flag, rank, fb, bs,
               (const T *)wb[cur], wb[1 - cur], (const int32_t *)lb[cur], lb[1 - cur]);
        cur ^= 1;
        launch(k_ls_next, nblk(ns + 1, T_), T_, 0, st, S, ns, nst, nn, nflag);
        cub::DeviceScan::ExclusiveSum(tmp, tb, nflag, nidx, 2 * ns + 1, st);
        launch(k_ls_owner_next<T>, nblk(M, T_), T_, 0, st, M, owner, S, (const int32_t *)nflag,
               (const int32_t *)nidx, (const T *)wb[cur], W, (const int32_t *)lb[cur], lab);
        cub::DeviceSelect::Flagged(tmp, tb, nst, nflag, S.start, cnt, 2 * ns, st);
        cub::DeviceSelect::Flagged(tmp, tb, nn, nflag, S.n, cnt, 2 * ns, st);
        RSG_CHECK_LAUNCH();
        RSG_CUDA(cudaMemcpyAsync(&ns, cnt, 4, cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
    }
    ar.used = mark;
}

}  // namespace rsg
