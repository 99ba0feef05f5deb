// Batched find_subs: every FOF group of a call is processed together, level
// by level of the 6D phase-space FOF hierarchy (src/groupies.c:520-708).
#pragma once
#include "halo_math.cuh"
#include "kdtree.cuh"

namespace rsg {

// Node of the subgroup hierarchy (a "subfof" of src/groupies.c:36-37):
// level 0 is the FOF group itself.  Arrays are indexed by global node id.
struct HierNodes {
    int32_t *start, *n, *parent, *group, *level, *nchild;
    int32_t *h0, *h1;      // halos created in the node's subtree
    int32_t *maxi, *ng;    // biggest halo, number of growing halos
    float *target_r;       // 6D linking length (normalised units)
    int32_t cap;
};

struct SubsOut {
    int64_t nhalos;
};

// Device-resident batched find_subs.
//  d_p      : caller particles (num_p), permuted in place on return
//  goff/gsz : groups (host arrays, ng groups); groups must not overlap
//  d_halos/d_extra : outputs (capacity max_halos)
//  exact    : 1 = the reference's labels, orders and sums (plain drop-in);
//             0 = batched mode (parallel labels and reductions)
SubsOut find_subs_device(Arena &ar, rsg_particle *d_p, int64_t num_p, const int64_t *goff,
                         const int64_t *gsz, int64_t ngroups, const rsg_config &cfg,
                         rsg_halo *d_halos, rsg_extra_halo_info *d_extra, int64_t max_halos,
                         cudaStream_t st, int exact);

}  // namespace rsg
