// Host driver of the level-synchronous kd-forest build (see kdtree.cuh).
#pragma once
#include "kdtree.cuh"

namespace rsg {

struct ToI64 {
    __device__ int64_t operator()(int32_t v) const { return (int64_t)v; }
};
// Fails with RSG_ERR_LIMIT when the int32 counts in[0..n) add up to more
// than an int32 offset can address: the callers scan such counts into
// int32 offsets.
inline void check_i32_total(Arena &ar, const int32_t *in, int64_t n, const char *what,
                            cudaStream_t st) {
    thrust::transform_iterator<ToI64, const int32_t *, int64_t> it(in, ToI64{});
    size_t mark = ar.used;
    int64_t *tot = ar.get<int64_t>(1);
    size_t b = 0;
    cub::DeviceReduce::Sum(nullptr, b, it, tot, (int)n, st);
    void *t = ar.take(b + 256);
    cub::DeviceReduce::Sum(t, b, it, tot, (int)n, st);
    RSG_CHECK_LAUNCH();
    int64_t h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, tot, sizeof(h), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    ar.used = mark;
    if (h > (int64_t)0x7fffffff - 1) {
        set_error(RSG_ERR_LIMIT, "%s: %lld entries exceed the 2^31 limit of one call", what,
                  (long long)h);
        throw Failure();
    }
}

// Box accumulation with per-thread runs: each thread walks ITEMS consecutive
// elements, keeps a running min/max while the owner stays the same and
// flushes with ordered atomics when it changes, so a node spanning millions
// of elements receives one atomic per run rather than one per element.
template <int D, class RecT, int ITEMS>
__global__ void k_box_runs(const RecT *recs, int64_t nrec, const int32_t *owner,
                           unsigned *bmin, unsigned *bmax) {
    int64_t i0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) * ITEMS;
    int cur = -1;
    unsigned lo[D], hi[D];
    for (int it = 0; it < ITEMS; it++) {
        int64_t i = i0 + it;
        if (i >= nrec) break;
        int a = owner[i];
        if (a != cur) {
            if (cur >= 0)
                for (int d = 0; d < D; d++) {
                    atomicMin(&bmin[(int64_t)cur * D + d], lo[d]);
                    atomicMax(&bmax[(int64_t)cur * D + d], hi[d]);
                }
            cur = a;
            for (int d = 0; d < D; d++) {
                lo[d] = 0xffffffffu;
                hi[d] = 0u;
            }
        }
        if (a < 0) continue;
        const RecT r = recs[i];
        for (int d = 0; d < D; d++) {
            unsigned o = f2ord(PosOf<RecT, D>::get(r, d));
            lo[d] = min(lo[d], o);
            hi[d] = max(hi[d], o);
        }
    }
    // last run: a warp whose lanes all hold the same node (the top levels of
    // a build) combines it first and issues one atomic per dimension
    const unsigned FULL = 0xffffffffu;
    if (__match_any_sync(FULL, cur) == FULL) {
        if (cur >= 0)
            for (int d = 0; d < D; d++) {
                unsigned a = __reduce_min_sync(FULL, lo[d]), b = __reduce_max_sync(FULL, hi[d]);
                if ((threadIdx.x & 31) == 0) {
                    atomicMin(&bmin[(int64_t)cur * D + d], a);
                    atomicMax(&bmax[(int64_t)cur * D + d], b);
                }
            }
    } else if (cur >= 0) {
        for (int d = 0; d < D; d++) {
            atomicMin(&bmin[(int64_t)cur * D + d], lo[d]);
            atomicMax(&bmax[(int64_t)cur * D + d], hi[d]);
        }
    }
}

template <int D>
__global__ void k_box_final_range(KNode<D> *nodes, int32_t first, int32_t count,
                                  const unsigned *bmin, const unsigned *bmax) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    int a = first + k;
    for (int d = 0; d < D; d++) {
        nodes[a].mn[d] = ord2f(bmin[(int64_t)a * D + d]);
        nodes[a].mx[d] = ord2f(bmax[(int64_t)a * D + d]);
    }
}

// The same for the last level's new nodes [ls->base, + ls->nnew), grid over ub.
template <int D>
__global__ void k_box_final_lvl(KNode<D> *nodes, const LevelState *ls, int32_t ub,
                                const unsigned *bmin, const unsigned *bmax) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ub || k >= ls->nnew) return;
    int a = ls->base + k;
    for (int d = 0; d < D; d++) {
        nodes[a].mn[d] = ord2f(bmin[(int64_t)a * D + d]);
        nodes[a].mx[d] = ord2f(bmax[(int64_t)a * D + d]);
    }
}
__global__ void k_iota_i32(int32_t *a, int32_t n);
#define RSG_FOREST_BATCH 4  // levels between reads of the build state

__global__ void k_root_owner(const int32_t *rstart, const int32_t *rn, int32_t ntrees,
                             int leaf, int32_t *owner, int32_t *box_owner);

template <int D>
__global__ void k_root_active(const KNode<D> *nodes, int32_t ntrees, int leaf, int32_t *flag) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntrees) return;
    flag[t] = nodes[t].n > leaf ? 1 : 0;
}

template <int D, class RecT>
Forest<D> build_forest(Arena &ar, RecT *recs, int64_t nrec, const int32_t *rstart,
                       const int32_t *rn, int32_t ntrees, int64_t n_in_trees, int leaf,
                       cudaStream_t st) {
    Forest<D> F;
    F.ntrees = ntrees;
    if (ntrees == 0) return F;
    const int T = 256;
    int64_t cap = ntrees + 4 * (n_in_trees / (leaf > 1 ? leaf : 1)) + 4096;
    if (cap > 2 * n_in_trees + ntrees + 16) cap = 2 * n_in_trees + ntrees + 16;
    KNode<D> *nodes = ar.get<KNode<D>>(cap);
    const size_t mark = ar.used;  // everything below is released on return
    unsigned *bmin = ar.get<unsigned>(cap * D), *bmax = ar.get<unsigned>(cap * D);
    int32_t *owner = ar.get<int32_t>(nrec), *box_owner = ar.get<int32_t>(nrec);
    RecT *tmp = ar.get<RecT>(nrec);
    int32_t *flag = ar.get<int32_t>(nrec + 1), *rank = ar.get<int32_t>(nrec + 1);
    int32_t *fb = ar.get<int32_t>(nrec), *bs = ar.get<int32_t>(nrec);
    int32_t *act = ar.get<int32_t>(cap), *act2 = ar.get<int32_t>(cap), *slot = ar.get<int32_t>(cap);
    float *lim = ar.get<float>(cap);
    int32_t *m_arr = ar.get<int32_t>(cap), *q_arr = ar.get<int32_t>(cap);
    int64_t *sflag = ar.get<int64_t>(cap + 1), *soff = ar.get<int64_t>(cap + 1);
    int32_t *nflag = ar.get<int32_t>(cap), *ids = ar.get<int32_t>(cap);
    LevelState *ls = ar.get<LevelState>(1);
    int32_t *lvl_end = ar.get<int32_t>(RSG_FOREST_LEVELS + 2);
    size_t cub_bytes = 0, b2 = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, cub_bytes, flag, rank, (int)(nrec + 1), st);
    cub::DeviceScan::ExclusiveSum(nullptr, b2, sflag, soff, (int)(cap + 1), st);
    cub_bytes = cub_bytes > b2 ? cub_bytes : b2;
    cub::DeviceSelect::Flagged(nullptr, b2, ids, nflag, act, &ls->nact, (int)cap, st);
    cub_bytes = cub_bytes > b2 ? cub_bytes : b2;
    void *cub_tmp = ar.take(cub_bytes + 256);

    launch(k_root_init<D, RecT>, nblk(ntrees, T), T, 0, st, rstart, rn, ntrees, nodes, bmin, bmax);
    RSG_CUDA(cudaMemsetAsync(owner, 0xff, sizeof(int32_t) * nrec, st));
    RSG_CUDA(cudaMemsetAsync(box_owner, 0xff, sizeof(int32_t) * nrec, st));
    {
        int64_t avg = n_in_trees / ntrees, y = avg / 2048;
        dim3 g((unsigned)ntrees, (unsigned)(y < 1 ? 1 : (y > 4096 ? 4096 : y)));
        launch(k_root_owner, g, 256, 0, st, rstart, rn, ntrees, leaf, owner, box_owner);
    }
    RSG_CHECK_LAUNCH();
    const int IT = 8;
    launch(k_box_runs<D, RecT, IT>, nblk((nrec + IT - 1) / IT, T), T, 0, st, recs, nrec, box_owner,
                                                                         bmin, bmax);
    launch(k_box_final_range<D>, nblk(ntrees, T), T, 0, st, nodes, 0, ntrees, bmin, bmax);
    launch(k_root_active<D>, nblk(ntrees, T), T, 0, st, nodes, ntrees, leaf, nflag);
    launch(k_iota_i32, nblk(ntrees, T), T, 0, st, ids, ntrees);
    {
        LevelState h0 = {};
        h0.nnodes = ntrees;
        RSG_CUDA(cudaMemcpyAsync(ls, &h0, sizeof(h0), cudaMemcpyHostToDevice, st));
    }
    cub::DeviceSelect::Flagged(cub_tmp, cub_bytes, ids, nflag, act, &ls->nact, ntrees, st);
    RSG_CHECK_LAUNCH();
    LevelState hs;
    RSG_CUDA(cudaMemcpyAsync(&hs, ls, sizeof(hs), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    F.level_end(0);
    F.level_end(ntrees);
    // Levels run back to back with their counts on the device; the host reads
    // the state every RSG_FOREST_BATCH levels.  Grids are sized by an upper
    // bound of the active count (ub): at most twice the previous level's,
    // and at most one active node per leaf + 1 records plus the roots.
    const int64_t amax = n_in_trees / (leaf + 1) + ntrees;
    int64_t ub = hs.nact;
    int level = 0;
    RecT *buf[2] = {recs, tmp};  // levels scatter back and forth between these
    int cur = 0;
    while (hs.nact > 0) {
        for (int b = 0; b < RSG_FOREST_BATCH && ub > 0; b++) {
            if (++level > RSG_FOREST_LEVELS) {
                set_error(RSG_ERR_LIMIT, "kd-forest build exceeded %d levels", RSG_FOREST_LEVELS);
                throw Failure();
            }
            const int32_t u = (int32_t)ub;
            launch(k_slot_set, nblk(u, T), T, 0, st, (const int32_t *)act, (const LevelState *)ls,
                   slot);
            launch(k_prep<D>, nblk(u, T), T, 0, st, nodes, (const int32_t *)act,
                   (const LevelState *)ls, lim);
            launch(k_flags<D, RecT>, nblk(nrec + 1, T), T, 0, st, (const RecT *)buf[cur], nrec,
                   owner, slot, nodes, lim, flag);
            cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, flag, rank, (int)(nrec + 1), st);
            launch(k_counts<D>, nblk(u, T), T, 0, st, nodes, (const int32_t *)act,
                   (const LevelState *)ls, rank, m_arr, q_arr);
            launch(k_tables<D>, nblk(nrec, T), T, 0, st, nodes, nrec, owner, slot, flag, rank,
                   m_arr, fb, bs);
            launch(k_scatter<D, RecT>, nblk(nrec, T), T, 0, st, nodes, (const RecT *)buf[cur],
                   buf[1 - cur], nrec, owner, slot, flag, rank, m_arr, q_arr, fb, bs);
            cur ^= 1;
            launch(k_split_flags<D>, nblk(u + 1, T), T, 0, st, m_arr, nodes, (const int32_t *)act,
                   (const LevelState *)ls, u, leaf, sflag);
            cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, sflag, soff, u + 1, st);
            RSG_CHECK_LAUNCH();
            launch(k_children<D>, nblk(u, T), T, 0, st, nodes, (const int32_t *)act, ls, m_arr,
                   (const int64_t *)soff, (int32_t)cap, leaf, act2, bmin, bmax);
            launch(k_level_advance, 1, 32, 0, st, ls, (const int64_t *)soff, lvl_end, level - 1);
            std::swap(act, act2);  // the next level's active nodes
            launch(k_owner_update<D, RecT>, nblk(nrec, T), T, 0, st, nodes, nrec, owner,
                   box_owner, leaf, (const RecT *)buf[cur], recs);
            launch(k_box_runs<D, RecT, IT>, nblk((nrec + IT - 1) / IT, T), T, 0, st,
                   (const RecT *)buf[cur], nrec, box_owner, bmin, bmax);
            const int64_t u2 = std::min<int64_t>(2 * ub, cap);
            launch(k_box_final_lvl<D>, nblk(u2, T), T, 0, st, nodes, (const LevelState *)ls,
                   (int32_t)u2, bmin, bmax);
            RSG_CHECK_LAUNCH();
            ub = std::min<int64_t>(u2, amax);
        }
        RSG_CUDA(cudaMemcpyAsync(&hs, ls, sizeof(hs), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        if (hs.err) {
            set_error(RSG_ERR_LIMIT, "kd-forest node capacity %lld exceeded", (long long)cap);
            throw Failure();
        }
        ub = hs.nact;
    }
    if (level > 0) {
        std::vector<int32_t> le(level);
        RSG_CUDA(cudaMemcpyAsync(le.data(), lvl_end, sizeof(int32_t) * level,
                                 cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        for (int l = 0; l < level; l++) F.level_end(le[l]);
    }
    const int32_t nnodes = hs.nnodes;
    F.nodes = nodes;
    F.nnodes = nnodes;
    ar.used = mark;
    return F;
}

}  // namespace rsg
