// Exact union-find labels from event lists (see uflabels.cuh).
#include <cub/cub.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "uflabels.cuh"

namespace rsg {

// "never" / "no candidate": the value a 0x7f byte fill gives, above any index
#define RSG_UF_NONE 0x7f7f7f7f

// ---- pointer doubling to the creating event --------------------------------
__global__ void k_uf_jump(int32_t *ptr, int64_t M, int *changed) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= M) return;
    int p = ptr[k];
    if (p < 0) return;
    int pp = ptr[p];
    if (pp != p) {
        ptr[k] = pp;  // an ancestor, whatever the order of the writes
        *changed = 1;
    }
}
__global__ void k_uf_newflag(const int32_t *ptr, int64_t M, int32_t *nf) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k > M) return;
    nf[k] = (k < M && ptr[k] == (int32_t)k) ? 1 : 0;
}
__global__ void k_uf_sfid(const int32_t *ptr, int64_t M, const int32_t *nsc, int32_t *sfid) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= M) return;
    int p = ptr[k];
    sfid[k] = p < 0 ? -1 : nsc[p];
}

int64_t uf_resolve(Arena &ar, int32_t *ptr, int64_t M, int32_t *sfid, int32_t *nsc,
                   cudaStream_t st) {
    const int T = 256;
    size_t mark = ar.used;
    int *changed = ar.get<int>(1);
    for (int round = 0;; round++) {
        if (round > 64) {
            set_error(RSG_ERR_LIMIT, "label pointer doubling did not converge");
            throw Failure();
        }
        RSG_CUDA(cudaMemsetAsync(changed, 0, sizeof(int), st));
        launch(k_uf_jump, nblk(M, T), T, 0, st, ptr, M, changed);
        launch(k_uf_jump, nblk(M, T), T, 0, st, ptr, M, changed);
        RSG_CHECK_LAUNCH();
        int h = 0;
        RSG_CUDA(cudaMemcpyAsync(&h, changed, sizeof(int), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        if (!h) break;
    }
    int32_t *nf = ar.get<int32_t>(M + 1);
    launch(k_uf_newflag, nblk(M + 1, T), T, 0, st, ptr, M, nf);
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, nf, nsc, (int)(M + 1), st);
    void *t = ar.take(b + 256);
    cub::DeviceScan::ExclusiveSum(t, b, nf, nsc, (int)(M + 1), st);
    launch(k_uf_sfid, nblk(M, T), T, 0, st, (const int32_t *)ptr, M, (const int32_t *)nsc, sfid);
    RSG_CHECK_LAUNCH();
    int32_t S = 0;
    RSG_CUDA(cudaMemcpyAsync(&S, nsc + M, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    ar.used = mark;
    return S;
}

// ---- Boruvka spanning forest of the candidate merges -----------------------
__global__ void k_bv_init(int32_t *comp, int64_t S) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v < S) comp[v] = (int32_t)v;
}
// compS[v] = the current root of v.  comp is a forest of hooks; path
// halving only ever replaces a pointer by an ancestor, so concurrent walks
// stay valid.
__global__ void k_bv_flatten(int32_t *comp, int64_t S, int32_t *compS) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= S) return;
    int x = (int)v;
    while (true) {
        int p = comp[x], gp = comp[p];
        if (p == gp) {
            compS[v] = p;
            return;
        }
        comp[x] = gp;
        x = gp;
    }
}
__global__ void k_bv_best(const int32_t *cF, const int32_t *cW, int64_t nc, const int32_t *compS,
                          int32_t *best, int *any) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) return;
    int a = compS[cF[c]], b = compS[cW[c]];
    if (a == b) return;
    atomicMin(&best[a], (int32_t)c);
    atomicMin(&best[b], (int32_t)c);
    *any = 1;
}
// Every root hooks onto the other side of its earliest outgoing merge; of
// two roots that chose the same merge the larger hooks (weights are
// distinct, so no longer cycle forms).
__global__ void k_bv_hook(const int32_t *cF, const int32_t *cW, const int32_t *compS,
                          const int32_t *best, int64_t S, int32_t *comp, uint8_t *msf) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= S || compS[v] != (int32_t)v) return;
    int c = best[v];
    if (c == RSG_UF_NONE) return;
    msf[c] = 1;
    int a = compS[cF[c]], b = compS[cW[c]];
    int other = (a == (int)v) ? b : a;
    if (best[other] == c && (int)v < other) return;
    comp[v] = other;
}
__global__ void k_bv_keys(const int32_t *eid, int32_t ne, const int32_t *cF, const int32_t *compS,
                          int32_t *key) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ne) key[t] = compS[cF[eid[t]]];
}
__global__ void k_bv_runflag(const int32_t *key, int32_t ne, int32_t *flag) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ne) flag[t] = (t == 0 || key[t] != key[t - 1]) ? 1 : 0;
}
__device__ __forceinline__ int rt_find(int32_t *R, int a) {
    int r = a;
    while (R[r] != r) r = R[r];
    while (R[a] != r) {
        int nx = R[a];
        R[a] = r;
        a = nx;
    }
    return r;
}
// One component per thread: its spanning merges in time order, each keeping
// the root of the link's set (merge_smallfofs, src/fof.c:72-90).  Components
// with more than RSG_UF_WARP merges are k_uf_replay_w's.
#define RSG_UF_WARP 64
__global__ void k_uf_replay(const int32_t *eid, const int32_t *rs, int32_t nr, int32_t ne,
                            const int32_t *cF, const int32_t *cW, int32_t *R) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nr) return;
    int e1 = (t + 1 < nr) ? rs[t + 1] : ne;
    if (e1 - rs[t] > RSG_UF_WARP) return;
    for (int i = rs[t]; i < e1; i++) {
        int c = eid[i];
        int rl = rt_find(R, cW[c]), rc = rt_find(R, cF[c]);
        if (rl != rc) R[rc] = rl;
    }
}
// The large components: one warp per component, 32 merges at a time.  The
// lanes find the roots of their merge's two sets in the state before the
// batch, in parallel; then the merges are applied in time order, lane by
// lane.  A root that an earlier merge of the batch ended is replaced by the
// root it was joined to (one forward pass over the batch's merges resolves a
// chain: a replacement can only be ended by a later merge), and a merge of
// two different sets makes W's root the parent of F's, as the sequential
// replay does.
#define RSG_UF_WARPS 4
__global__ void __launch_bounds__(RSG_UF_WARPS * 32)
    k_uf_replay_w(const int32_t *eid, const int32_t *rs, int32_t nr, int32_t ne,
                  const int32_t *cF, const int32_t *cW, int32_t *R) {
    __shared__ int32_t killed_s[RSG_UF_WARPS][32], into_s[RSG_UF_WARPS][32];
    const unsigned FULL = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= nr) return;
    const int e0 = rs[t], e1 = (t + 1 < nr) ? rs[t + 1] : ne;
    if (e1 - e0 <= RSG_UF_WARP) return;
    int32_t *killed = killed_s[w], *into = into_s[w];
    for (int b = e0; b < e1; b += 32) {
        const int i = b + lane;
        int rl = -1, rc = -1;
        if (i < e1) {
            const int c = eid[i];
            rl = rt_find(R, cW[c]);
            rc = rt_find(R, cF[c]);
        }
        __syncwarp();
        const int m = min(32, e1 - b);
        int nk = 0;
        for (int q = 0; q < m; q++) {
            int done = 0;
            if (lane == q) {
                for (int k = 0; k < nk; k++) {
                    if (rl == killed[k]) rl = into[k];
                    if (rc == killed[k]) rc = into[k];
                }
                if (rl != rc) {
                    R[rc] = rl;
                    killed[nk] = rc;
                    into[nk] = rl;
                    done = 1;
                }
            }
            nk += __shfl_sync(FULL, done, q);
            __syncwarp();
        }
    }
}
__global__ void k_uf_rootall(int32_t *R, int64_t S, int32_t *root) {
    int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (v >= S) return;
    int r = (int)v;
    while (R[r] != r) r = R[r];
    root[v] = r;
}

template <class It>
static int32_t sel_flagged(Arena &ar, It in, const int32_t *flag, int32_t *out, int64_t n,
                           cudaStream_t st) {
    size_t mark = ar.used;
    int *cnt = ar.get<int>(1);
    size_t b = 0;
    cub::DeviceSelect::Flagged(nullptr, b, in, flag, out, cnt, (int)n, st);
    void *t = ar.take(b + 256);
    cub::DeviceSelect::Flagged(t, b, in, flag, out, cnt, (int)n, st);
    RSG_CHECK_LAUNCH();
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    ar.used = mark;
    return h;
}
__global__ void k_u8_to_i32(const uint8_t *a, int64_t n, int32_t *b) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

void uf_roots(Arena &ar, const int32_t *cF, const int32_t *cW, int64_t nc, int64_t S,
              int32_t *root, cudaStream_t st) {
    const int T = 256;
    if (S <= 0) return;
    if (nc >= RSG_UF_NONE || S >= RSG_UF_NONE) {
        set_error(RSG_ERR_LIMIT, "too many label merges (%lld) or sets (%lld)", (long long)nc,
                  (long long)S);
        throw Failure();
    }
    size_t mark = ar.used;
    int32_t *R = ar.get<int32_t>(S);
    launch(k_bv_init, nblk(S, T), T, 0, st, R, S);
    if (nc > 0) {
        int32_t *comp = ar.get<int32_t>(S), *compS = ar.get<int32_t>(S), *best = ar.get<int32_t>(S);
        uint8_t *msf = ar.get<uint8_t>(nc);
        int *any = ar.get<int>(1);
        RSG_CUDA(cudaMemsetAsync(msf, 0, nc, st));
        launch(k_bv_init, nblk(S, T), T, 0, st, comp, S);
        for (int round = 0;; round++) {
            if (round > 64) {
                set_error(RSG_ERR_LIMIT, "spanning forest rounds did not converge");
                throw Failure();
            }
            launch(k_bv_flatten, nblk(S, T), T, 0, st, comp, S, compS);
            RSG_CUDA(cudaMemcpyAsync(comp, compS, 4 * S, cudaMemcpyDeviceToDevice, st));
            RSG_CUDA(cudaMemsetAsync(best, 0x7f, 4 * S, st));  // RSG_UF_NONE
            RSG_CUDA(cudaMemsetAsync(any, 0, sizeof(int), st));
            launch(k_bv_best, nblk(nc, T), T, 0, st, cF, cW, nc, (const int32_t *)compS, best, any);
            RSG_CHECK_LAUNCH();
            int h = 0;
            RSG_CUDA(cudaMemcpyAsync(&h, any, sizeof(int), cudaMemcpyDeviceToHost, st));
            RSG_CUDA(cudaStreamSynchronize(st));
            if (!h) break;
            launch(k_bv_hook, nblk(S, T), T, 0, st, cF, cW, (const int32_t *)compS,
                   (const int32_t *)best, S, comp, msf);
        }
        // compS: final components; the spanning merges, grouped by component
        // with time order kept inside (stable sort on the component)
        int32_t *mflag = ar.get<int32_t>(nc), *eid = ar.get<int32_t>(nc);
        launch(k_u8_to_i32, nblk(nc, T), T, 0, st, (const uint8_t *)msf, nc, mflag);
        thrust::counting_iterator<int32_t> it(0);
        size_t m2 = ar.used;
        int *cnt = ar.get<int>(1);
        size_t b = 0;
        cub::DeviceSelect::Flagged(nullptr, b, it, mflag, eid, cnt, (int)nc, st);
        void *tb = ar.take(b + 256);
        cub::DeviceSelect::Flagged(tb, b, it, mflag, eid, cnt, (int)nc, st);
        int32_t ne = 0;
        RSG_CUDA(cudaMemcpyAsync(&ne, cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        RSG_CUDA(cudaStreamSynchronize(st));
        ar.used = m2;
        if (ne > 0) {
            int32_t *key = ar.get<int32_t>(ne), *key2 = ar.get<int32_t>(ne);
            int32_t *eid2 = ar.get<int32_t>(ne);
            launch(k_bv_keys, nblk(ne, T), T, 0, st, (const int32_t *)eid, ne, cF,
                   (const int32_t *)compS, key);
            int bits = 1;
            while (bits < 31 && ((int64_t)1 << bits) < S) bits++;
            size_t sb = 0;
            cub::DeviceRadixSort::SortPairs(nullptr, sb, key, key2, eid, eid2, ne, 0, bits, st);
            void *stb = ar.take(sb + 256);
            cub::DeviceRadixSort::SortPairs(stb, sb, key, key2, eid, eid2, ne, 0, bits, st);
            int32_t *rflag = ar.get<int32_t>(ne), *rs = ar.get<int32_t>(ne);
            launch(k_bv_runflag, nblk(ne, T), T, 0, st, (const int32_t *)key2, ne, rflag);
            int32_t nr = sel_flagged(ar, thrust::counting_iterator<int32_t>(0), rflag, rs, ne, st);
            launch(k_uf_replay, nblk(nr, 64), 64, 0, st, (const int32_t *)eid2, (const int32_t *)rs,
                   nr, ne, cF, cW, R);
            launch(k_uf_replay_w, nblk((int64_t)nr * 32, RSG_UF_WARPS * 32), RSG_UF_WARPS * 32, 0,
                   st, (const int32_t *)eid2, (const int32_t *)rs, nr, ne, cF, cW, R);
        }
    }
    launch(k_uf_rootall, nblk(S, T), T, 0, st, R, S, root);
    RSG_CHECK_LAUNCH();
    ar.used = mark;
}

// ---- the 6D form over CSR lists of later neighbours ------------------------
__global__ void k_el_g(const int32_t *eln, int64_t M, const int32_t *noff, const int32_t *nbr,
                       int32_t *g) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= M || eln[k] < 0) return;
    int e0 = noff[k], e1 = noff[k + 1];
    if (e0 == e1) return;
    atomicMin(&g[k], (int32_t)k);
    for (int e = e0; e < e1; e++) atomicMin(&g[nbr[e]], (int32_t)k);
}
// f(k): the set of k (labelled earlier), else that of the first later
// neighbour labelled earlier, else a new one (src/fof.c:116-131).
__global__ void k_el_ptr(const int32_t *eln, int64_t M, const int32_t *noff, const int32_t *nbr,
                         const int32_t *g, int32_t *ptr) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= M) return;
    int p = -1;
    if (eln[k] >= 0) {
        int e0 = noff[k], e1 = noff[k + 1];
        if (e0 < e1) {
            int gk = g[k];
            if (gk < (int)k) {
                p = gk;
            } else {
                p = (int)k;
                for (int e = e0; e < e1; e++) {
                    int gj = g[nbr[e]];
                    if (gj < (int)k) {
                        p = gj;
                        break;
                    }
                }
            }
        }
    }
    ptr[k] = p;
}
__global__ void k_el_lab0(const int32_t *g, int64_t M, const int32_t *sfid, int32_t *lab0) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= M) return;
    int gj = g[j];
    lab0[j] = (gj == RSG_UF_NONE) ? -1 : sfid[gj];
}
// Candidate merges of event k: the labels of its later neighbours labelled
// before k that differ from f(k), first occurrence of each (a later repeat
// of a label meets the same set and changes nothing); MODE 0 counts, 1
// fills.  Both passes skip the same entries.
#define RSG_UF_SEEN 8
template <int MODE>
__global__ void k_el_cand(const int32_t *eln, int64_t M, const int32_t *noff, const int32_t *nbr,
                          const int32_t *g, const int32_t *lab0, const int32_t *sfid,
                          const int32_t *coff, int32_t *ccnt, int32_t *cF, int32_t *cW) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= M) return;
    int cnt = 0;
    if (eln[k] >= 0) {
        int e0 = noff[k], e1 = noff[k + 1];
        if (e0 < e1) {
            int F = sfid[k];
            int seen[RSG_UF_SEEN];
            int ns = 0;
            int o = MODE ? coff[k] : 0;
            for (int e = e0; e < e1; e++) {
                int j = nbr[e];
                if (g[j] >= (int)k) continue;
                int W = lab0[j];
                if (W == F) continue;
                bool dup = false;
                for (int q = 0; q < ns; q++) dup |= (seen[q] == W);
                if (dup) continue;
                if (ns < RSG_UF_SEEN) seen[ns++] = W;
                if (MODE) {
                    cF[o + cnt] = F;
                    cW[o + cnt] = W;
                }
                cnt++;
            }
        }
    }
    if (!MODE) ccnt[k] = cnt;
}
__global__ void k_el_final(const int32_t *eln, int64_t M, const int32_t *nstart,
                           const int32_t *lab0, const int32_t *root, const int32_t *nsc,
                           int32_t *lab) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= M) return;
    int k = eln[j];
    if (k < 0) return;
    int l = lab0[j];
    lab[j] = (l < 0) ? -1 : root[l] - nsc[nstart[k]];
}

void exact_labels_csr(Arena &ar, int64_t M, const int32_t *eln, const int32_t *nstart,
                      const int32_t *noff, const int32_t *nbr, int32_t *lab, cudaStream_t st) {
    const int T = 256;
    if (M <= 0) return;
    size_t mark = ar.used;
    int32_t *g = ar.get<int32_t>(M), *ptr = ar.get<int32_t>(M), *sfid = ar.get<int32_t>(M);
    int32_t *nsc = ar.get<int32_t>(M + 1), *lab0 = ar.get<int32_t>(M);
    RSG_CUDA(cudaMemsetAsync(g, 0x7f, 4 * M, st));  // RSG_UF_NONE: never labelled
    launch(k_el_g, nblk(M, T), T, 0, st, eln, M, noff, nbr, g);
    launch(k_el_ptr, nblk(M, T), T, 0, st, eln, M, noff, nbr, (const int32_t *)g, ptr);
    RSG_CHECK_LAUNCH();
    int64_t S = uf_resolve(ar, ptr, M, sfid, nsc, st);
    launch(k_el_lab0, nblk(M, T), T, 0, st, (const int32_t *)g, M, (const int32_t *)sfid, lab0);
    int32_t *ccnt = ar.get<int32_t>(M + 1), *coff = ar.get<int32_t>(M + 1);
    RSG_CUDA(cudaMemsetAsync(ccnt + M, 0, sizeof(int32_t), st));
    launch(k_el_cand<0>, nblk(M, T), T, 0, st, eln, M, noff, nbr, (const int32_t *)g,
           (const int32_t *)lab0, (const int32_t *)sfid, (const int32_t *)nullptr, ccnt,
           (int32_t *)nullptr, (int32_t *)nullptr);
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, ccnt, coff, (int)(M + 1), st);
    size_t m1 = ar.used;
    void *t = ar.take(b + 256);
    cub::DeviceScan::ExclusiveSum(t, b, ccnt, coff, (int)(M + 1), st);
    ar.used = m1;
    RSG_CHECK_LAUNCH();
    int32_t nc = 0;
    RSG_CUDA(cudaMemcpyAsync(&nc, coff + M, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    int32_t *cF = ar.get<int32_t>(nc + 1), *cW = ar.get<int32_t>(nc + 1);
    launch(k_el_cand<1>, nblk(M, T), T, 0, st, eln, M, noff, nbr, (const int32_t *)g,
           (const int32_t *)lab0, (const int32_t *)sfid, (const int32_t *)coff, ccnt, cF, cW);
    int32_t *root = ar.get<int32_t>(S + 1);
    uf_roots(ar, cF, cW, nc, S, root, st);
    launch(k_el_final, nblk(M, T), T, 0, st, eln, M, nstart, (const int32_t *)lab0,
           (const int32_t *)root, (const int32_t *)nsc, lab);
    RSG_CHECK_LAUNCH();
    ar.used = mark;
}

}  // namespace rsg
