// Particle input: a GADGET-2 snapshot file into particle records, and the id
// sort of the particles before halo finding, with the records assembled and
// sorted on the device.
//   rsg_read_gadget2[_device]          load_particles_gadget2
//                                      (src/io/io_gadget.c:200-254) with
//                                      gadget2_detect_filetype (:17-39),
//                                      gadget2_read_stride (:41-120),
//                                      gadget2_extract_header_info (:122-179)
//                                      and gadget2_rescale_particles (:181-198)
//   rsg_sort_particles_by_id[_device]  std::sort of p by id
//                                      (src/mpi_main.cpp:2021-2024)
// The host parses the file's small records (Fortran record markers, the
// optional block tags of the GADGET variants, the header, either byte order)
// and finds where the position, velocity and id payloads lie; those go to the
// device straight from the file through the pinned staging threads
// (hoststage.cuh), where one kernel swaps bytes, widens ids, narrows double
// coordinates and applies the unit conversions into the reference's particle
// records.
#include <errno.h>
#include <fcntl.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cub/cub.cuh>
#include <vector>

#include "common.cuh"
#include "hoststage.cuh"

namespace rsg {
Arena &call_arena(size_t bytes, cudaStream_t *st);  // api.cu
namespace {

const double kCriticalDensity = 2.77519737e11;  // src/universal_constants.h:5

// struct gadget_header (src/io/io_gadget.h:8-27), 256 bytes
struct GHeader {
    uint32_t npart[6];
    double mass[6];
    double time, redshift;
    int32_t flag_sfr, flag_feedback;
    uint32_t npart_total[6];
    int32_t flag_cooling, num_files;
    double box, om, ol, h0;
    int32_t flag_stellarage, flag_metals;
    int32_t npart_total_hw[6];
    int32_t flag_entropy_ics;
    char unused[256 - 8 * 12 - 4 * 13 - 4 * 12];
};
static_assert(sizeof(GHeader) == 256, "GADGET header is 256 bytes");

uint32_t bswap32(uint32_t v) {
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}
void swap_words(void *p, size_t bytes) {
    uint32_t *w = (uint32_t *)p;
    for (size_t i = 0; i < bytes / 4; i++) w[i] = bswap32(w[i]);
}
void swap_halves(double *d) {
    uint32_t w[2];
    memcpy(w, d, 8);
    uint32_t t = w[0];
    w[0] = w[1];
    w[1] = t;
    memcpy(d, w, 8);
}

struct Reader {
    int fd = -1;
    int64_t off = 0, size = 0;  // read position and file size
    bool swap = false;
    const char *path;
    ~Reader() {
        if (fd >= 0) close(fd);
    }
    void fail(const char *what) {
        set_error(RSG_ERR_IO, "rsg_read_gadget2: %s in %s", what, path);
        throw Failure();
    }
    void open_file() {
        fd = open(path, O_RDONLY);
        struct stat sb;
        if (fd < 0 || fstat(fd, &sb) != 0) fail("cannot open");
        size = (int64_t)sb.st_size;
    }
    void read(void *p, size_t n) {
        size_t got = 0;
        while (got < n) {
            const ssize_t r = pread(fd, (char *)p + got, n - got, (off_t)(off + (int64_t)got));
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) fail("file is truncated");
            got += (size_t)r;
        }
        off += (int64_t)n;
    }
    uint32_t word() {
        uint32_t v;
        read(&v, 4);
        return swap ? bswap32(v) : v;
    }
    // a region of n bytes that must lie inside the file; returns its offset
    int64_t span(int64_t n) {
        if (n < 0 || off + n > size) fail("file is truncated");
        const int64_t at = off;
        off += n;
        return at;
    }
    // a whole Fortran record of at most `n` bytes (head and tail markers
    // equal, src/io/io_util.c:53-84)
    void record(void *p, size_t n) {
        const uint32_t head = word();
        if (head > n) fail("record longer than expected");
        read(p, head);
        if (word() != head) fail("record markers differ");
        if (head < n) memset((char *)p + head, 0, n - head);
    }
    // the block tag of the GADGET variants ("HEAD", "POS", ...)
    void tag(int variant, const char *want) {
        if (!variant) return;
        char t[8] = {0};
        record(t, 4 * (size_t)variant);
        if (strncmp(t, want, strlen(want)) != 0) fail("unexpected block tag");
    }
};

// raw blocks -> particle records
__global__ void k_gadget_assemble(const unsigned char *pos, const unsigned char *vel,
                                  const unsigned char *ids, int64_t n, int cw, int iw, int swap,
                                  double conv, double vres, rsg_particle *out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    rsg_particle q;
    for (int blk = 0; blk < 2; blk++) {
        const unsigned char *src = (blk ? vel : pos) + (size_t)i * 3 * cw;
        for (int j = 0; j < 3; j++) {
            float v;
            if (cw == 4) {
                uint32_t w;
                memcpy(&w, src + 4 * j, 4);
                if (swap) w = __byte_perm(w, 0, 0x0123);
                v = __uint_as_float(w);
            } else {
                uint32_t lo, hi;
                memcpy(&lo, src + 8 * j, 4);
                memcpy(&hi, src + 8 * j + 4, 4);
                if (swap) {
                    const uint32_t t = __byte_perm(lo, 0, 0x0123);
                    lo = __byte_perm(hi, 0, 0x0123);
                    hi = t;
                }
                v = (float)__hiloint2double((int)hi, (int)lo);
            }
            // float *= double: the product in double, rounded to float
            q.pos[blk * 3 + j] = (float)((double)v * (blk ? vres : conv));
        }
    }
    if (iw == 4) {
        uint32_t w;
        memcpy(&w, ids + (size_t)i * 4, 4);
        if (swap) w = __byte_perm(w, 0, 0x0123);
        q.id = (int64_t)w;  // a 4-byte id is unsigned (src/io/io_gadget.c:187-191)
    } else {
        uint32_t lo, hi;
        memcpy(&lo, ids + (size_t)i * 8, 4);
        memcpy(&hi, ids + (size_t)i * 8 + 4, 4);
        if (swap) {
            const uint32_t t = __byte_perm(lo, 0, 0x0123);
            lo = __byte_perm(hi, 0, 0x0123);
            hi = t;
        }
        q.id = (int64_t)(((uint64_t)hi << 32) | lo);
    }
    out[i] = q;
}

// smallest and largest id (ordered atomics on the signed values)
__global__ void k_id_range(const rsg_particle *p, int64_t n, long long *mm) {
    long long lo = LLONG_MAX, hi = LLONG_MIN;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const long long v = (long long)p[i].id;
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
    for (int o = 16; o; o >>= 1) {
        const long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hi);
    }
}
// keys id - min as unsigned (order-preserving for signed ids), values the
// record index
__global__ void k_id_keys(const rsg_particle *p, int64_t n, const long long *mm,
                          unsigned long long *key, int32_t *idx) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = (unsigned long long)p[i].id - (unsigned long long)mm[0];
    idx[i] = (int32_t)i;
}
__global__ void k_gather_p(const rsg_particle *src, const int32_t *idx, int64_t n,
                           rsg_particle *dst) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}
__global__ void k_mm_init(long long *mm) {
    mm[0] = LLONG_MAX;
    mm[1] = LLONG_MIN;
}

}  // namespace
}  // namespace rsg

namespace rsg {
namespace {

// One file into records at out_dev (device) or out_host (host): the body of
// rsg_read_gadget2 and rsg_read_gadget2_device.
int read_core(const char *path, const struct rsg_gadget_opts *opt, struct rsg_config *cfg,
              struct rsg_particle *out_host, struct rsg_particle *out_dev, int64_t max_p,
              int64_t *num_p) {
    struct rsg_particle *want = out_host ? out_host : out_dev;
    if (!path || !opt || !cfg || !num_p || max_p < 0 || (max_p && !want) ||
        opt->halo_particle_type < 0 || opt->halo_particle_type > 5) {
        set_error(RSG_ERR_ARGS, "rsg_read_gadget2: bad arguments");
        return RSG_ERR_ARGS;
    }
    try {
        Reader R;
        R.path = path;
        R.open_file();
        // gadget2_detect_filetype: the first record marker is 256 (no tags),
        // 4 or 8 (tagged variants), in this machine's byte order or not
        uint32_t first;
        R.read(&first, 4);
        if (first != 4 && first != 256 && first != 8) {
            R.swap = true;
            first = bswap32(first);
        }
        const int variant = first == 4 ? 1 : first == 8 ? 2 : first == 256 ? 0 : -1;
        if (variant < 0) R.fail("unrecognised GADGET2 file type");
        R.off = 0;
        GHeader h;
        R.tag(variant, "HEAD");
        R.record(&h, sizeof h);
        if (R.swap) {  // every 4-byte word, then the halves of each double
            swap_words(&h, sizeof h);
            for (int i = 0; i < 6; i++) swap_halves(&h.mass[i]);
            swap_halves(&h.time);
            swap_halves(&h.redshift);
            swap_halves(&h.box);
            swap_halves(&h.om);
            swap_halves(&h.ol);
            swap_halves(&h.h0);
        }
        // gadget2_extract_header_info
        if (fabs(h.om + h.ol - 1.0) > 1e-5) {
            set_error(RSG_ERR_INPUT, "rsg_read_gadget2: curved cosmology (Om %f, Ol %f) in %s", h.om,
                      h.ol, path);
            return RSG_ERR_INPUT;
        }
        const int t = (int)opt->halo_particle_type;
        cfg->ol = h.ol;
        cfg->om = h.om;
        cfg->h0 = h.h0;
        cfg->box_size = h.box * opt->length_conversion;
        int64_t total = ((int64_t)h.npart_total_hw[t] << 32) + (int64_t)h.npart_total[t];
        if (opt->lgadget && t < 5)
            total = ((int64_t)h.npart_total[t + 1] << 32) + (int64_t)h.npart_total[t];
        cfg->total_particles = total;
        cfg->scale_now = h.time;
        if (h.mass[t] || !cfg->particle_mass || opt->rescale_particle_mass) {
            if (!opt->rescale_particle_mass)
                cfg->particle_mass = h.mass[t] * opt->mass_conversion;
            else
                cfg->particle_mass =
                    cfg->om * kCriticalDensity * pow(cfg->box_size, 3) / (double)total;
        }
        cfg->avg_particle_spacing = cbrt(cfg->particle_mass / (cfg->om * kCriticalDensity));
        // the particles of the halo type, or all of them
        int64_t all = 0, skip = 0, keep, skip2;
        for (int i = 0; i < 6; i++) all += h.npart[i];
        if (opt->skip_non_halo) {
            for (int i = 0; i < t; i++) skip += h.npart[i];
            keep = h.npart[t];
            skip2 = all - skip - keep;
        } else {
            keep = all;
            skip2 = 0;
        }
        *num_p = keep;
        if (!want) return 0;  // the count alone
        if (keep > max_p) {
            set_error(RSG_ERR_ARGS, "rsg_read_gadget2: %lld particles for %lld places",
                      (long long)keep, (long long)max_p);
            return RSG_ERR_ARGS;
        }
        // gadget2_read_stride for POS, VEL and ID: the element width from the
        // record length, the other types' elements skipped; the payload of
        // the kept particles is located here and read by the staging threads
        struct Block {
            int width;
            int64_t at, bytes;
        };
        auto block = [&](const char *name, int stride) {
            R.tag(variant, name);
            const uint32_t len = R.word();
            const int64_t elems = (int64_t)stride * (skip + keep + skip2);
            Block b;
            if ((int64_t)len == elems * 4) b.width = 4;
            else if ((int64_t)len == elems * 8) b.width = 8;
            else R.fail("block size does not match the particle counts");
            R.span(skip * stride * b.width);
            b.bytes = keep * stride * b.width;
            b.at = R.span(b.bytes);
            R.span(skip2 * stride * b.width);
            if (R.word() != len) R.fail("record markers differ");
            return b;
        };
        const Block bp = block("POS", 3), bv = block("VEL", 3), bi = block("ID", 1);
        if (bp.width != bv.width) R.fail("positions and velocities differ in width");
        if (keep == 0) return 0;
        cudaStream_t st;
        Arena &ar = call_arena((size_t)(bp.bytes + bv.bytes + bi.bytes) +
                                   (out_host ? sizeof(rsg_particle) * (size_t)keep : 0) +
                                   (64u << 20),
                               &st);
        unsigned char *d_pos = ar.get<unsigned char>(bp.bytes), *d_vel = ar.get<unsigned char>(bv.bytes);
        unsigned char *d_id = ar.get<unsigned char>(bi.bytes);
        rsg_particle *d_out = out_host ? ar.get<rsg_particle>(keep) : out_dev;
        stage_h2d({{R.fd, bp.at, nullptr, d_pos, (size_t)bp.bytes},
                   {R.fd, bv.at, nullptr, d_vel, (size_t)bv.bytes},
                   {R.fd, bi.at, nullptr, d_id, (size_t)bi.bytes}},
                  path);
        const double vres = opt->lightcone ? 1.0 : sqrt(cfg->scale_now);
        launch(k_gadget_assemble, nblk(keep, 256), 256, 0, st, (const unsigned char *)d_pos,
               (const unsigned char *)d_vel, (const unsigned char *)d_id, keep, bp.width, bi.width,
               (int)R.swap, opt->length_conversion, vres, d_out);
        RSG_CHECK_LAUNCH();
        RSG_CUDA(cudaStreamSynchronize(st));
        if (out_host) stage_d2h(out_host, d_out, sizeof(rsg_particle) * (size_t)keep);
        return 0;
    } catch (Failure &) {
        return error_code();
    }
}

// d_p[0..n) sorted by id on the device (stable radix sort of id - min over
// the bits the id range needs, then a gather of the records)
void sort_device(rsg_particle *d_p, int64_t n, Arena &ar, cudaStream_t st) {
    rsg_particle *d_q = ar.get<rsg_particle>(n);
    unsigned long long *k1 = ar.get<unsigned long long>(n), *k2 = ar.get<unsigned long long>(n);
    int32_t *v1 = ar.get<int32_t>(n), *v2 = ar.get<int32_t>(n);
    long long *mm = ar.get<long long>(2);
    launch(k_mm_init, 1, 1, 0, st, mm);
    launch(k_id_range, 152 * 8, 256, 0, st, (const rsg_particle *)d_p, n, mm);
    RSG_CHECK_LAUNCH();
    long long h_mm[2];
    RSG_CUDA(cudaMemcpyAsync(h_mm, mm, sizeof h_mm, cudaMemcpyDeviceToHost, st));
    RSG_CUDA(cudaStreamSynchronize(st));
    if (h_mm[0] == h_mm[1]) return;  // one id: the order stays
    const unsigned long long range = (unsigned long long)h_mm[1] - (unsigned long long)h_mm[0];
    const int end_bit = 64 - __builtin_clzll(range);
    launch(k_id_keys, nblk(n, 256), 256, 0, st, (const rsg_particle *)d_p, n,
           (const long long *)mm, k1, v1);
    size_t tb = 0;
    RSG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, k1, k2, v1, v2, (int)n, 0, end_bit, st));
    void *tmp = ar.take(tb + 256);
    RSG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, k1, k2, v1, v2, (int)n, 0, end_bit, st));
    launch(k_gather_p, nblk(n, 256), 256, 0, st, (const rsg_particle *)d_p, (const int32_t *)v2,
           n, d_q);
    RSG_CHECK_LAUNCH();
    RSG_CUDA(cudaMemcpyAsync(d_p, d_q, sizeof(rsg_particle) * (size_t)n, cudaMemcpyDeviceToDevice,
                             st));
    RSG_CUDA(cudaStreamSynchronize(st));
}

const size_t kSortBytesPerRec = sizeof(rsg_particle) + 2 * 8 + 2 * 4 + 32;

}  // namespace
}  // namespace rsg

using namespace rsg;

extern "C" int rsg_read_gadget2(const char *path, const struct rsg_gadget_opts *opt,
                                struct rsg_config *cfg, struct rsg_particle *p, int64_t max_p,
                                int64_t *num_p) {
    return read_core(path, opt, cfg, p, nullptr, max_p, num_p);
}

extern "C" int rsg_read_gadget2_device(const char *path, const struct rsg_gadget_opts *opt,
                                       struct rsg_config *cfg, struct rsg_particle *d_p,
                                       int64_t max_p, int64_t *num_p) {
    return read_core(path, opt, cfg, nullptr, d_p, max_p, num_p);
}

extern "C" int rsg_sort_particles_by_id(struct rsg_particle *p, int64_t n) {
    if (n < 0 || (n && !p) || n >= ((int64_t)1 << 31)) {
        set_error(RSG_ERR_ARGS, "rsg_sort_particles_by_id: bad arguments");
        return RSG_ERR_ARGS;
    }
    if (n < 2) return 0;
    try {
        cudaStream_t st;
        Arena &ar = call_arena((size_t)n * (sizeof(rsg_particle) + kSortBytesPerRec) + (64u << 20), &st);
        rsg_particle *d_p = ar.get<rsg_particle>(n);
        stage_h2d({{-1, 0, p, d_p, sizeof(rsg_particle) * (size_t)n}}, nullptr);
        sort_device(d_p, n, ar, st);
        stage_d2h(p, d_p, sizeof(rsg_particle) * (size_t)n);
        return 0;
    } catch (Failure &) {
        return error_code();
    }
}

extern "C" int rsg_sort_particles_by_id_device(struct rsg_particle *d_p, int64_t n) {
    if (n < 0 || (n && !d_p) || n >= ((int64_t)1 << 31)) {
        set_error(RSG_ERR_ARGS, "rsg_sort_particles_by_id_device: bad arguments");
        return RSG_ERR_ARGS;
    }
    if (n < 2) return 0;
    try {
        cudaStream_t st;
        Arena &ar = call_arena((size_t)n * kSortBytesPerRec + (64u << 20), &st);
        sort_device(d_p, n, ar, st);
        return 0;
    } catch (Failure &) {
        return error_code();
    }
}
