// Pinned, multi-threaded host <-> device staging (hoststage.cuh).
#include <errno.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <thread>

#include "common.cuh"
#include "hoststage.cuh"

namespace rsg {
namespace {

constexpr size_t kChunk = 8u << 20;  // bytes per chunk and per pinned slot
constexpr int kMaxWorkers = 8;

// The calling thread's slots and streams (two pinned slots per worker).
struct Pool {
    int nw = 0, dev = -1;
    void *slot[kMaxWorkers][2] = {};
    cudaStream_t st[kMaxWorkers] = {};
    cudaEvent_t ev[kMaxWorkers][2] = {};
    void release() {
        for (int w = 0; w < kMaxWorkers; w++) {
            for (int s = 0; s < 2; s++) {
                if (slot[w][s]) cudaFreeHost(slot[w][s]);
                if (ev[w][s]) cudaEventDestroy(ev[w][s]);
                slot[w][s] = nullptr;
                ev[w][s] = nullptr;
            }
            if (st[w]) cudaStreamDestroy(st[w]);
            st[w] = nullptr;
        }
        nw = 0;
        dev = -1;
    }
    ~Pool() { release(); }
};
thread_local Pool t_pool;

Pool &pool() {
    int dev;
    RSG_CUDA(cudaGetDevice(&dev));
    Pool &P = t_pool;
    if (P.nw && P.dev == dev) return P;
    P.release();
    const unsigned hc = std::thread::hardware_concurrency();
    const int nw = std::max(1, std::min(kMaxWorkers, hc ? (int)hc : 4));
    for (int w = 0; w < nw; w++) {
        for (int s = 0; s < 2; s++) {
            cudaError_t e = cudaHostAlloc(&P.slot[w][s], kChunk, cudaHostAllocDefault);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P.ev[w][s], cudaEventDisableTiming);
            if (e != cudaSuccess) {
                P.release();
                set_error(RSG_ERR_CUDA, "staging slots: %s", cudaGetErrorString(e));
                throw Failure();
            }
        }
        cudaError_t e = cudaStreamCreateWithFlags(&P.st[w], cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            P.release();
            set_error(RSG_ERR_CUDA, "staging streams: %s", cudaGetErrorString(e));
            throw Failure();
        }
    }
    P.nw = nw;
    P.dev = dev;
    return P;
}

// First failure of any worker; the others stop at their next chunk.
struct Shared {
    std::atomic<size_t> next{0};
    std::atomic<int> failed{0};
    std::mutex mu;
    int code = 0;
    std::string msg;
    void fail(int c, const std::string &m) {
        std::lock_guard<std::mutex> g(mu);
        if (!code) {
            code = c;
            msg = m;
        }
        failed = 1;
    }
    void cuda(cudaError_t e, const char *where) {
        fail(RSG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
    }
};

// Runs fn(0..n-1), worker 0 on the calling thread.  If a thread cannot be
// started the remaining workers are simply not run: the shared chunk counter
// hands their chunks to the others.
template <class F>
void run_workers(int n, F fn) {
    std::vector<std::thread> th;
    for (int w = 1; w < n; w++) {
        try {
            th.emplace_back(fn, w);
        } catch (...) {
            break;
        }
    }
    fn(0);
    for (auto &t : th) t.join();
}

struct Chunk {
    const HostPiece *p;
    size_t off, bytes;
};

void h2d_worker(Pool &P, int w, const std::vector<Chunk> &ch, Shared &S) {
    cudaError_t e = cudaSetDevice(P.dev);
    if (e != cudaSuccess) return S.cuda(e, "cudaSetDevice");
    bool pending[2] = {false, false};
    for (int k = 0; !S.failed; k++) {
        const size_t c = S.next.fetch_add(1);
        if (c >= ch.size()) break;
        const int s = k & 1;
        if (pending[s] && (e = cudaEventSynchronize(P.ev[w][s])) != cudaSuccess) {
            S.cuda(e, "cudaEventSynchronize");
            break;
        }
        const Chunk &C = ch[c];
        char *slot = (char *)P.slot[w][s];
        if (C.p->fd >= 0) {
            size_t got = 0;
            while (got < C.bytes) {
                const ssize_t r = pread(C.p->fd, slot + got, C.bytes - got,
                                        (off_t)(C.p->off + (int64_t)(C.off + got)));
                if (r < 0 && errno == EINTR) continue;
                if (r <= 0) break;
                got += (size_t)r;
            }
            if (got < C.bytes) {
                S.fail(RSG_ERR_IO, "file is truncated");
                break;
            }
        } else {
            memcpy(slot, (const char *)C.p->src + C.off, C.bytes);
        }
        e = cudaMemcpyAsync((char *)C.p->dst + C.off, slot, C.bytes, cudaMemcpyHostToDevice,
                            P.st[w]);
        if (e == cudaSuccess) e = cudaEventRecord(P.ev[w][s], P.st[w]);
        if (e != cudaSuccess) {
            S.cuda(e, "cudaMemcpyAsync");
            break;
        }
        pending[s] = true;
    }
    if ((e = cudaStreamSynchronize(P.st[w])) != cudaSuccess) S.cuda(e, "cudaStreamSynchronize");
}

void d2h_worker(Pool &P, int w, char *dst, const char *src, size_t total, size_t nch, Shared &S) {
    cudaError_t e = cudaSetDevice(P.dev);
    if (e != cudaSuccess) return S.cuda(e, "cudaSetDevice");
    int64_t prev = -1;
    int prev_s = 0;
    bool ok = true;
    // copy the chunk the slot holds out to dst, once its transfer is done
    auto drain = [&](int64_t c, int s) {
        cudaError_t e2 = cudaEventSynchronize(P.ev[w][s]);
        if (e2 != cudaSuccess) {
            S.cuda(e2, "cudaEventSynchronize");
            ok = false;
            return;
        }
        const size_t off = (size_t)c * kChunk;
        memcpy(dst + off, P.slot[w][s], std::min(kChunk, total - off));
    };
    for (int k = 0; ok && !S.failed; k++) {
        const size_t c = S.next.fetch_add(1);
        if (c >= nch) break;
        const int s = k & 1;  // its previous chunk was drained in the last iteration
        const size_t off = c * kChunk;
        e = cudaMemcpyAsync(P.slot[w][s], src + off, std::min(kChunk, total - off),
                            cudaMemcpyDeviceToHost, P.st[w]);
        if (e == cudaSuccess) e = cudaEventRecord(P.ev[w][s], P.st[w]);
        if (e != cudaSuccess) {
            S.cuda(e, "cudaMemcpyAsync");
            ok = false;
            break;
        }
        if (prev >= 0) drain(prev, prev_s);
        prev = (int64_t)c;
        prev_s = s;
    }
    if (ok && prev >= 0) drain(prev, prev_s);
    if ((e = cudaStreamSynchronize(P.st[w])) != cudaSuccess) S.cuda(e, "cudaStreamSynchronize");
}

void rethrow(Shared &S, const char *what) {
    if (!S.code) return;
    if (S.code == RSG_ERR_IO)
        set_error(RSG_ERR_IO, "%s in %s", S.msg.c_str(), what ? what : "(input)");
    else
        set_error(S.code, "staging: %s", S.msg.c_str());
    throw Failure();
}

}  // namespace

void stage_h2d(const std::vector<HostPiece> &pieces, const char *what) {
    std::vector<Chunk> ch;
    for (const HostPiece &p : pieces)
        for (size_t off = 0; off < p.bytes; off += kChunk)
            ch.push_back({&p, off, std::min(kChunk, p.bytes - off)});
    if (ch.empty()) return;
    Pool &P = pool();
    Shared S;
    const int n = (int)std::min<size_t>((size_t)P.nw, ch.size());
    run_workers(n, [&](int w) { h2d_worker(P, w, ch, S); });
    rethrow(S, what);
}

void stage_d2h(void *dst, const void *src, size_t bytes) {
    if (!bytes) return;
    Pool &P = pool();
    Shared S;
    const size_t nch = (bytes + kChunk - 1) / kChunk;
    const int n = (int)std::min<size_t>((size_t)P.nw, nch);
    run_workers(n, [&](int w) {
        d2h_worker(P, w, (char *)dst, (const char *)src, bytes, nch, S);
    });
    rethrow(S, nullptr);
}

void read_file_parallel(int fd, int64_t off, void *dst, size_t bytes, const char *what) {
    if (!bytes) return;
    const size_t nch = (bytes + kChunk - 1) / kChunk;
    const unsigned hc = std::thread::hardware_concurrency();
    const int n = (int)std::min<size_t>((size_t)std::max(1, std::min(kMaxWorkers, hc ? (int)hc : 4)),
                                        nch);
    Shared S;
    run_workers(n, [&](int) {
        while (!S.failed) {
            const size_t c = S.next.fetch_add(1);
            if (c >= nch) break;
            const size_t o = c * kChunk, b = std::min(kChunk, bytes - o);
            size_t got = 0;
            while (got < b) {
                const ssize_t r = pread(fd, (char *)dst + o + got, b - got,
                                        (off_t)(off + (int64_t)(o + got)));
                if (r < 0 && errno == EINTR) continue;
                if (r <= 0) break;
                got += (size_t)r;
            }
            if (got < b) S.fail(RSG_ERR_IO, "file is truncated");
        }
    });
    rethrow(S, what);
}

namespace {
// pageable host memory of at least four chunks: worth the staging threads
bool staged(const void *h, size_t bytes) {
    if (bytes < 4 * kChunk) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();  // clear the error the query recorded
        return false;
    }
    return a.type == cudaMemoryTypeUnregistered;
}
}  // namespace

void host_to_device(void *d, const void *h, size_t bytes, cudaStream_t st) {
    if (!bytes) return;
    if (!staged(h, bytes)) {
        RSG_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
        return;
    }
    RSG_CUDA(cudaStreamSynchronize(st));  // d may still be read by earlier work
    stage_h2d({{-1, 0, h, d, bytes}}, nullptr);
}

void device_to_host(void *h, const void *d, size_t bytes, cudaStream_t st) {
    if (!bytes) return;
    if (!staged(h, bytes)) {
        RSG_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st));
        return;
    }
    RSG_CUDA(cudaStreamSynchronize(st));  // the producing work ends first
    stage_d2h(h, d, bytes);
}

}  // namespace rsg
