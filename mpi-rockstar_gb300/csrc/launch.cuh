// Every kernel of the library is launched through launch(): it skips empty
// grids, counts launches (reported by rsg_launch_count) and, for the one
// kernel selected with rsg_profile_select, brackets each launch with CUDA
// events on the launching stream so its device time can be read back.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

namespace rsg {

struct LaunchStats {
    int64_t launches = 0;
    bool selecting = false;  // a kernel name is selected for event timing
};
LaunchStats &launch_stats();
bool prof_match(const void *func);
void prof_begin(cudaStream_t st, const void *func);
void prof_end(cudaStream_t st);

template <class... KA, class... A>
inline void launch(void (*k)(KA...), dim3 g, dim3 b, size_t sm, cudaStream_t st, A &&...a) {
    if (g.x == 0 || g.y == 0 || g.z == 0) return;
    LaunchStats &S = launch_stats();
    bool prof = S.selecting && prof_match((const void *)k);
    if (prof) prof_begin(st, (const void *)k);
    k<<<g, b, sm, st>>>(std::forward<A>(a)...);
    S.launches++;
    if (prof) prof_end(st);
}

}  // namespace rsg
