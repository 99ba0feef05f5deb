// Host <-> device transfers of large host buffers and file regions through
// pinned staging slots, filled and drained by several host threads at once.
//
// A copy from pageable memory (a file read into a heap buffer, a caller's
// particle array) is bound by one host thread's memcpy and by the driver's
// own staging.  Here the transfer is cut into chunks; each worker thread owns
// two pinned slots and a stream, fills one slot (pread from the file, or
// memcpy from host memory) while the other one's cudaMemcpyAsync is in
// flight, and takes the next chunk from a shared counter.  The slots and
// streams belong to the calling thread and are made once.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include <cuda_runtime.h>

namespace rsg {

// One contiguous region of a host-to-device transfer.
struct HostPiece {
    int fd;           // >= 0: the bytes are read from this file at `off`
    int64_t off;      // file offset (fd >= 0)
    const void *src;  // fd < 0: the bytes are copied from here
    void *dst;        // device destination
    size_t bytes;
};

// Every piece copied to the device; returns once all copies have completed.
// A short read fails with RSG_ERR_IO (`what` names the file in the message),
// a CUDA failure with RSG_ERR_CUDA (both throw Failure, as RSG_CUDA does).
void stage_h2d(const std::vector<HostPiece> &pieces, const char *what);

// dst[0..bytes) (any host memory) <- src (device); returns when done.
void stage_d2h(void *dst, const void *src, size_t bytes);

// bytes of file fd from offset off into host memory dst, by up to eight
// threads reading 8 MiB chunks with pread (no device involved); a short read
// fails with RSG_ERR_IO naming `what`.
void read_file_parallel(int fd, int64_t off, void *dst, size_t bytes, const char *what);

// A caller's host buffer to or from the device around work on stream st.
// Page-locked memory, and buffers of a few chunks, are copied with
// cudaMemcpyAsync on st; larger pageable buffers go through the staging
// threads, after st has been synchronised, and are complete on return.
void host_to_device(void *d, const void *h, size_t bytes, cudaStream_t st);
void device_to_host(void *h, const void *d, size_t bytes, cudaStream_t st);

}  // namespace rsg
