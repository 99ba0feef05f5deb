// Exact union-find labels of the reference's FOF linking without replaying
// the links one after another.
//
// link_particle_to_fof / link_fof_to_fof / merge_smallfofs (src/fof.c:46-170)
// visit events in order (one per processed particle; a 3D seed adds a second
// one for its 2r sphere).  A label, once given, never changes, and a merge
// keeps the root of the link's set.  Written as functions of the event lists:
//   g(j)   = the first linking event (>= 2 entries) whose list holds j: the
//            moment j receives its label;
//   f(k)   = the set event k works on: the label of k if g(k) < k, else the
//            label of the first j of its list with g(j) < k, else a new
//            smallfof (creation rank = index among creating events);
//            resolved to the creating event by pointer doubling;
//   merges = for every j of an event's list labelled before the event, a
//            candidate (F = f(k), W = label of j) in event/list order.
// The final root of a component is the result of applying its merges in
// time order, each one keeping the root of W's set.  Only the merges that
// join two different sets matter, and those are exactly the minimum spanning
// forest of the candidates weighted by time (Kruskal's order is time order),
// which Boruvka rounds find in parallel.  Each component then replays its
// own spanning edges -- about 2% of its particles -- in time order.
#pragma once
#include "common.cuh"

namespace rsg {

// Resolves ptr (event -> event whose set it uses, itself for a creating
// event, -1 for no event) to the creating event, numbers the creating events
// in index order and writes, for every event k, sfid[k] = the smallfof
// number of its set and, for every index, nsc[k] = the number of creating
// events before k (nsc has M + 1 entries).  Returns the number of smallfofs.
int64_t uf_resolve(Arena &ar, int32_t *ptr, int64_t M, int32_t *sfid, int32_t *nsc,
                   cudaStream_t st);

// Final root smallfof of every smallfof v < S (root[v]) from the candidate
// merges (cF[c], cW[c]), c = 0..nc-1 in time order: Boruvka spanning forest,
// then each component's spanning merges applied in time order, each keeping
// the root of W's set (src/fof.c:72-90).
void uf_roots(Arena &ar, const int32_t *cF, const int32_t *cW, int64_t nc, int64_t S,
              int32_t *root, cudaStream_t st);

// The 6D form: events are the elements k with eln[k] >= 0 and a non-empty
// list of later neighbours nbr[noff[k] .. noff[k+1]) (the list of
// link_particle_to_fof is k itself followed by them, src/groupies.c:274-284
// with src/fast3tree.c:419-465).  Writes, for every element of the level's
// nodes, the label the reference's build_fullfofs sorts by: the node-local
// smallfof number of its final root, -1 for a particle never linked.
// nstart[eln[k]] is the first element of k's node.
void exact_labels_csr(Arena &ar, int64_t M, const int32_t *eln, const int32_t *nstart,
                      const int32_t *noff, const int32_t *nbr, int32_t *lab, cudaStream_t st);

}  // namespace rsg
