// 3D FOF of one bounded chunk that allocates no device memory: every
// scratch buffer of the device pipeline is carved from one fixed device
// array declared in this file, and the caller passes device buffers and a
// stream.  (The host side keeps a few small std::vector tables on the host
// heap; no call here allocates or frees device memory.  The seed frontiers
// of the 3D FOF, a device-side graph loop elsewhere, are driven from the
// host here, step by step: instantiating a graph may take device memory.)
//
// Who needs it: an in-situ caller -- halo finding run inside an N-body
// code's time step on the GPU that also holds the simulation -- owns the
// device memory it budgets for the run and keeps kernels in flight on its
// own streams.  cudaMalloc may fail once that budget is handed out, and
// cudaFree waits for the whole device, which would stall the simulation's
// streams at every call.  Such a caller cannot let the halo finder allocate
// or free; it can afford a fixed, known amount of memory taken once.
//
// Setup: every call looks up the scratch array's device address for the
// current device with cudaGetSymbolAddress, checks the return code and
// passes that address on; nothing is cached, so the address stays right
// when the caller resets the device or recreates its primary context.  The
// first call in a process (and again after such a reset) loads the
// library's kernels and the array itself, which takes device memory once;
// make that call at setup, before any stream capture begins.  Later calls
// take no device memory.  The call synchronises its stream before it
// returns (it reads the group count back).
//
// Zero state: no part of the scratch has to start at zero.  Every buffer
// carved from it is written, or cleared with cudaMemsetAsync on the
// caller's stream, before it is read; the array keeps the last call's
// contents.
//
// Overlap: the scratch is one array per device, shared by every caller in
// the process.  Two calls that overlapped in time on one device would
// overwrite each other's buffers.  A call returns only after its stream has
// drained, so overlap can only come from host threads calling at once; a
// call that finds another in progress on its device returns RSG_ERR_BUSY
// and touches nothing.
#include <mutex>

#include "kdtree_impl.cuh"

namespace rsg {

struct FofOut {
    int64_t num_p;
    int64_t nfofs;
};
FofOut fof3d_device(Arena &ar, const rsg_particle *d_in, int64_t n, const rsg_config &cfg,
                    rsg_particle *d_out, int64_t *d_off, int64_t *d_sz, cudaStream_t st);

static __device__ __align__(256) char g_fof_scratch[RSG_NOALLOC_SCRATCH_BYTES];

#define RSG_NOALLOC_DEVICES 64
static std::mutex g_busy[RSG_NOALLOC_DEVICES];

// The scratch array's device address on the current device, looked up at
// every call (cheap once the module is loaded; never stale).
static int scratch_for_device(void **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_fof_scratch);
    if (e != cudaSuccess || !p) {
        set_error(RSG_ERR_CUDA, "rsg_rockstar_fof_noalloc: cudaGetSymbolAddress: %s",
                  cudaGetErrorString(e));
        return RSG_ERR_CUDA;
    }
    *out = p;
    return RSG_OK;
}

// An Arena over the fixed array: take() bumps inside it and fails with
// RSG_ERR_LIMIT when the chunk's buffers do not fit; nothing is freed.
struct BorrowedArena {
    Arena a;
    BorrowedArena(void *p, size_t bytes) {
        a.base = (char *)p;
        a.cap = bytes;
        a.fixed = true;
    }
    ~BorrowedArena() {
        a.base = nullptr;
        a.cap = 0;
    }
};

}  // namespace rsg

using namespace rsg;

extern "C" int rsg_rockstar_fof_noalloc(const struct rsg_particle *d_in, int64_t num_p,
                                        const struct rsg_config *cfg, struct rsg_particle *d_out,
                                        int64_t *num_p_out, int64_t *d_fof_offsets,
                                        int64_t *d_fof_sizes, int64_t max_fofs,
                                        int64_t *num_fofs, void *stream) {
    if (!cfg || !num_p_out || !num_fofs || num_p < 0 || max_fofs < 0 ||
        (num_p > 0 && (!d_in || !d_out)) || (max_fofs > 0 && (!d_fof_offsets || !d_fof_sizes))) {
        set_error(RSG_ERR_ARGS, "rsg_rockstar_fof_noalloc: null or negative argument");
        return RSG_ERR_ARGS;
    }
    if (num_p > RSG_NOALLOC_MAX_PARTICLES) {
        set_error(RSG_ERR_LIMIT,
                  "rsg_rockstar_fof_noalloc: %lld particles exceed its fixed limit of %d "
                  "(use rsg_rockstar_fof for larger sets)",
                  (long long)num_p, RSG_NOALLOC_MAX_PARTICLES);
        return RSG_ERR_LIMIT;
    }
    const char *a0 = (const char *)d_in, *b0 = (const char *)d_out;
    size_t bytes = sizeof(rsg_particle) * (size_t)num_p;
    if (num_p > 0 && a0 < b0 + bytes && b0 < a0 + bytes) {
        set_error(RSG_ERR_ARGS, "rsg_rockstar_fof_noalloc: d_in and d_out overlap");
        return RSG_ERR_ARGS;
    }
    *num_p_out = 0;
    *num_fofs = 0;
    if (num_p == 0) return RSG_OK;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        set_error(RSG_ERR_NO_DEVICE, "rsg_rockstar_fof_noalloc: no CUDA device available");
        return RSG_ERR_NO_DEVICE;
    }
    if (dev >= RSG_NOALLOC_DEVICES) {
        set_error(RSG_ERR_ARGS, "rsg_rockstar_fof_noalloc: device %d beyond the %d supported", dev,
                  RSG_NOALLOC_DEVICES);
        return RSG_ERR_ARGS;
    }
    std::unique_lock<std::mutex> busy(g_busy[dev], std::try_to_lock);
    if (!busy.owns_lock()) {
        set_error(RSG_ERR_BUSY, "rsg_rockstar_fof_noalloc: another call is using device %d's scratch",
                  dev);
        return RSG_ERR_BUSY;
    }
    void *scratch = nullptr;
    int rc = scratch_for_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    try {
        BorrowedArena B(scratch, RSG_NOALLOC_SCRATCH_BYTES);
        int64_t gcap = num_p / 2 + 1;  // groups hold >= 2 particles
        int64_t *s_off = B.a.get<int64_t>(gcap), *s_sz = B.a.get<int64_t>(gcap);
        FofOut o = fof3d_device(B.a, d_in, num_p, *cfg, d_out, s_off, s_sz, st);
        if (o.nfofs > max_fofs) {
            set_error(RSG_ERR_ARGS, "rsg_rockstar_fof_noalloc: %lld groups exceed max_fofs %lld",
                      (long long)o.nfofs, (long long)max_fofs);
            return RSG_ERR_ARGS;
        }
        if (o.nfofs) {
            RSG_CUDA(cudaMemcpyAsync(d_fof_offsets, s_off, sizeof(int64_t) * o.nfofs,
                                     cudaMemcpyDeviceToDevice, st));
            RSG_CUDA(cudaMemcpyAsync(d_fof_sizes, s_sz, sizeof(int64_t) * o.nfofs,
                                     cudaMemcpyDeviceToDevice, st));
        }
        RSG_CUDA(cudaStreamSynchronize(st));
        *num_p_out = o.num_p;
        *num_fofs = o.nfofs;
        return RSG_OK;
    } catch (Failure &) {
        // work already queued reads and writes the scratch: let it drain
        // before the next caller may take the array
        cudaStreamSynchronize(st);
        return error_code();
    }
}
