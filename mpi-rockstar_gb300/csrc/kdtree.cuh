// Level-synchronous kd-forest build on the GPU that reproduces, element for
// element, the in-place permutation of the reference's fast3tree build
// (src/fast3tree.c:736-908).
//
// The reference splits a node [0, n) at lim = 0.5f * (max + min) of its
// widest dimension with a two-pointer swap: a front pointer i walks up and,
// whenever p[i] > lim, swaps it with the back pointer j, which walks down.
// With m = #(p <= lim) the result is, in closed form:
//   * small elements before m stay put;
//   * the t-th big element before m (rank t, ascending) ends at n-1 (t = 0)
//     or one slot below the (t-1)-th small element after m counted from the
//     back;
//   * the t-th small element after m counted from the back fills the slot of
//     the t-th big element before m;
//   * big elements above the last consumed back position move down one;
//   * if the untouched tail [m, pos_last) holds two or more elements, it is
//     rotated down by one (the front pointer stops at m and swaps it with
//     each tail element in turn).
// Every element's destination is therefore a function of per-node prefix
// counts of the "big" flag, which one global scan provides for all nodes of
// a level at once.  Degenerate nodes (max == min on the split dimension) get
// lim = +inf so nothing moves, as in the reference's early return.
#pragma once
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/transform_iterator.h>

#include <vector>

#include "common.cuh"

namespace rsg {

template <class RecT, int D>
struct PosOf;
template <int D>
struct PosOf<Rec, D> {
    __device__ static float get(const Rec &r, int d) { return r.pos[d]; }
};

struct PotRec {  // struct potential (src/potential.h:7-21), 48 bytes
    float pos[6], r2;
    float pad;
    double pe;
    float ke;
    int32_t flags;
};
static_assert(sizeof(PotRec) == 48, "PotRec layout");
template <int D>
struct PosOf<PotRec, D> {
    __device__ static float get(const PotRec &r, int d) { return r.pos[d]; }
};

struct MetricRec {  // struct halo_metric (src/subhalo_metric.h): pos[4] + target
    float pos[4];
    int32_t target;
    int32_t pad[3];
};
template <int D>
struct PosOf<MetricRec, D> {
    __device__ static float get(const MetricRec &r, int d) { return r.pos[d]; }
};

#define RSG_FOREST_LEVELS 4096  // deepest build accepted (checked by build_forest)

// Device-side state of a forest build: the level's active count and the
// node bookkeeping, so that levels run back to back without a host round
// trip; the host reads it every few levels.
struct LevelState {
    int32_t nact;    // active nodes of the level being split
    int32_t nnodes;  // nodes created so far
    int32_t base;    // first node created by the last level
    int32_t nnew;    // nodes created by the last level
    int32_t err;     // node capacity exceeded
    int32_t pad[3];
};

template <int D>
struct Forest {
    KNode<D> *nodes = nullptr;  // nodes[t] is the root of tree t
    int32_t nnodes = 0;
    int32_t ntrees = 0;
    // nodes created by level l of the build are [lv_first[l], lv_first[l+1]),
    // l < nlv - 1; a fixed table so a build touches no host heap
    int32_t lv_first[RSG_FOREST_LEVELS + 2];
    int32_t nlv = 0;
    void level_end(int32_t first) { lv_first[nlv++] = first; }
};

// ---- kernels ------------------------------------------------------------

template <int D, class RecT>
__global__ void k_root_init(const int32_t *rstart, const int32_t *rn, int32_t ntrees,
                            KNode<D> *nodes, unsigned *bmin, unsigned *bmax) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntrees) return;
    KNode<D> &nd = nodes[t];
    nd.start = rstart[t];
    nd.n = rn[t];
    nd.div = -1;
    nd.left = -1;
    nd.parent = -1;
    nd.tree = t;
    for (int d = 0; d < D; d++) {
        bmin[t * D + d] = 0xffffffffu;
        bmax[t * D + d] = 0u;
    }
}


// Choose the split dimension and limit (src/fast3tree.c:736-757).
template <int D>
__global__ void k_prep(KNode<D> *nodes, const int32_t *act, const LevelState *ls, float *lim) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ls->nact) return;
    KNode<D> &nd = nodes[act[k]];
    int dim = D - 1;
    float dmax = fsub(nd.mx[D - 1], nd.mn[D - 1]);
    for (int i = 0; i < D - 1; i++) {
        float d2 = fsub(nd.mx[i], nd.mn[i]);
        if (d2 > dmax) {
            dmax = d2;
            dim = i;
        }
    }
    nd.div = dim;
    float l = fmul(0.5f, fadd(nd.mx[dim], nd.mn[dim]));
    if (nd.mx[dim] == nd.mn[dim]) l = __int_as_float(0x7f800000);  // +inf: nothing moves
    lim[k] = l;
}

template <int D, class RecT>
__global__ void k_flags(const RecT *recs, int64_t nrec, const int32_t *owner,
                        const int32_t *slot, const KNode<D> *nodes, const float *lim,
                        int32_t *flag) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i > nrec) return;
    int f = 0;
    if (i < nrec) {
        int a = owner[i];
        if (a >= 0) {
            int k = slot[a];
            f = PosOf<RecT, D>::get(recs[i], nodes[a].div) > lim[k];
        }
    }
    flag[i] = f;
}

// m (= #small) and q (= #big before m) per active node.
template <int D>
__global__ void k_counts(const KNode<D> *nodes, const int32_t *act, const LevelState *ls,
                         const int32_t *rank, int32_t *m_out, int32_t *q_out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ls->nact) return;
    const KNode<D> &nd = nodes[act[k]];
    int s = nd.start, n = nd.n;
    int B = rank[s + n] - rank[s];
    int m = n - B;
    m_out[k] = m;
    q_out[k] = rank[s + m] - rank[s];
}

template <int D>
__global__ void k_tables(const KNode<D> *nodes, int64_t nrec, const int32_t *owner,
                         const int32_t *slot, const int32_t *flag, const int32_t *rank,
                         const int32_t *m_arr, int32_t *fb, int32_t *bs) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nrec) return;
    int a = owner[i];
    if (a < 0) return;
    int k = slot[a];
    int s = nodes[a].start;
    int l = (int)(i - s);
    int br = rank[i] - rank[s];
    int sr = l - br;
    int m = m_arr[k];
    if (flag[i] && l < m) fb[s + br] = l;
    if (!flag[i] && l >= m) bs[s + (m - 1 - sr)] = l;
}

template <int D, class RecT>
__global__ void k_scatter(const KNode<D> *nodes, const RecT *src, RecT *dst, int64_t nrec,
                          const int32_t *owner, const int32_t *slot, const int32_t *flag,
                          const int32_t *rank, const int32_t *m_arr, const int32_t *q_arr,
                          const int32_t *fb, const int32_t *bs) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nrec) return;
    int a = owner[i];
    if (a < 0) return;
    int k = slot[a];
    int s = nodes[a].start, n = nodes[a].n;
    int l = (int)(i - s);
    int br = rank[i] - rank[s];
    int sr = l - br;
    int m = m_arr[k], q = q_arr[k];
    int big = flag[i];
    int d;
    if (!big && l < m) {
        d = l;
    } else if (big && l < m) {
        d = (br == 0) ? n - 1 : bs[s + br - 1] - 1;
    } else if (!big) {
        d = fb[s + (m - 1 - sr)];
    } else {
        int pos_last = (q > 0) ? bs[s + q - 1] : n;
        if (l > pos_last)
            d = l - 1;
        else if (pos_last - m >= 2)
            d = (l == m) ? pos_last - 1 : l - 1;
        else
            d = l;
    }
    dst[s + d] = src[i];
}


// Split bookkeeping (src/fast3tree.c:798-846): create children for nodes
// with 0 < m < n, turn the rest into leaves.  off[k] packs, over the active
// nodes before k, the splits (high 32 bits) and the children that split
// again (low 32 bits): node k's children go to nodes[ls->nnodes + 2 * splits]
// and those holding more than `leaf` records to next[children], which is the
// order a selection over the new nodes gives.  A level that would pass `cap`
// nodes sets ls->err and changes nothing.
template <int D>
__global__ void k_children(KNode<D> *nodes, const int32_t *act, LevelState *ls,
                           const int32_t *m_arr, const int64_t *off, int32_t cap, int leaf,
                           int32_t *next, unsigned *bmin, unsigned *bmax) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nact = ls->nact, base = ls->nnodes;
    if ((int64_t)base + 2 * (off[nact] >> 32) > cap) {
        if (k == 0) ls->err = 1;
        return;
    }
    if (k >= nact) return;
    int a = act[k];
    KNode<D> &nd = nodes[a];
    int m = m_arr[k];
    if (m == 0 || m == nd.n) {
        nd.div = -1;
        nd.left = -1;
        return;
    }
    int l = base + 2 * (int)(off[k] >> 32);
    int na = (int)(off[k] & 0xffffffffu);
    nd.left = l;
    if (m > leaf) next[na++] = l;
    if (nd.n - m > leaf) next[na] = l + 1;
    for (int c = 0; c < 2; c++) {
        KNode<D> &ch = nodes[l + c];
        ch.start = nd.start + (c ? m : 0);
        ch.n = c ? nd.n - m : m;
        ch.div = -1;
        ch.left = -1;
        ch.parent = a;
        ch.tree = nd.tree;
        for (int d = 0; d < D; d++) {
            bmin[(int64_t)(l + c) * D + d] = 0xffffffffu;
            bmax[(int64_t)(l + c) * D + d] = 0u;
        }
    }
}

// Element owner update: elements of split nodes move to their child.  The
// levels scatter between two buffers; an element whose node stops splitting
// is final now, and is copied from the buffer the level wrote (cur) to the
// output array (out) when they differ -- once per element, not once per level.
template <int D, class RecT>
__global__ void k_owner_update(const KNode<D> *nodes, int64_t nrec, int32_t *owner,
                               int32_t *box_owner, int leaf, const RecT *cur, RecT *out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nrec) return;
    int a = owner[i];
    if (a < 0) {
        box_owner[i] = -1;
        return;
    }
    const KNode<D> &nd = nodes[a];
    if (nd.left < 0) {
        owner[i] = -1;
        box_owner[i] = -1;
        if (cur != out) out[i] = cur[i];
        return;
    }
    int l = nd.left;
    int c = (i - nd.start) < nodes[l].n ? l : l + 1;
    box_owner[i] = c;
    bool fin = nodes[c].n <= leaf;
    owner[i] = fin ? -1 : c;
    if (fin && cur != out) out[i] = cur[i];
}

// sflag[0 .. ub]: per active node, split (high 32 bits) and children that
// split again (low 32 bits); 0 beyond the level's active count (ub bounds it
// from above).
template <int D>
__global__ void k_split_flags(const int32_t *m_arr, const KNode<D> *nodes, const int32_t *act,
                              const LevelState *ls, int32_t ub, int leaf, int64_t *sflag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > ub) return;
    if (k >= ls->nact) {
        sflag[k] = 0;
        return;
    }
    int m = m_arr[k], n = nodes[act[k]].n;
    int64_t v = 0;
    if (m > 0 && m < n) v = ((int64_t)1 << 32) | (int64_t)((m > leaf) + (n - m > leaf));
    sflag[k] = v;
}

__global__ void k_slot_set(const int32_t *act, const LevelState *ls, int32_t *slot);
__global__ void k_level_advance(LevelState *ls, const int64_t *off, int32_t *lvl_end,
                                int32_t level);

// Builds a kd-forest over recs[0..nrec) whose trees are the segments
// (rstart[t], rn[t]) (device arrays).  Elements outside every segment are
// left alone.  `recs` is permuted in place.  Returns the forest; node
// storage comes from the arena.
template <int D, class RecT>
Forest<D> build_forest(Arena &ar, RecT *recs, int64_t nrec, const int32_t *rstart,
                       const int32_t *rn, int32_t ntrees, int64_t n_in_trees, int leaf,
                       cudaStream_t st);

}  // namespace rsg
