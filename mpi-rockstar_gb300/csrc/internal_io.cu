// The reference's internal particle format (FILE_FORMAT "INTERNAL" for
// input; the DUMP_PARTICLES output): the 256-byte binary header with
// particle_type PARTICLE_TYPE_FULL, then the particle records verbatim.
//   rsg_read_internal[_device]  load_particles_internal
//                               (src/io/io_internal.c:85-100) with
//                               read_binary_header_config (:43-50)
//   rsg_write_internal          output_particles_internal (:52-83) for
//                               fraction 0 or 1 (every particle)
// The records need no conversion, so the host variant reads them straight
// into the caller's array with parallel preads and the device variant sends
// them from the page cache to HBM through the pinned staging threads.
#include <errno.h>
#include <fcntl.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#include "binheader.cuh"
#include "common.cuh"
#include "hoststage.cuh"

namespace rsg {
Arena &call_arena(size_t bytes, cudaStream_t *st);  // api.cu
namespace {

struct Fd {
    int fd = -1;
    ~Fd() {
        if (fd >= 0) close(fd);
    }
};

int read_core(const char *path, struct rsg_config *cfg, struct rsg_particle *out_host,
              struct rsg_particle *out_dev, int64_t max_p, int64_t *num_p) {
    struct rsg_particle *want = out_host ? out_host : out_dev;
    if (!path || !cfg || !num_p || max_p < 0 || (max_p && !want)) {
        set_error(RSG_ERR_ARGS, "rsg_read_internal: bad arguments");
        return RSG_ERR_ARGS;
    }
    try {
        if (out_dev) {  // the device variant needs a device first
            cudaStream_t st;
            call_arena(0, &st);
        }
        Fd F;
        F.fd = open(path, O_RDONLY);
        struct stat sb;
        if (F.fd < 0 || fstat(F.fd, &sb) != 0) {
            set_error(RSG_ERR_IO, "rsg_read_internal: cannot open %s", path);
            return RSG_ERR_IO;
        }
        BinHeader H;
        if (pread(F.fd, &H, sizeof H, 0) != (ssize_t)sizeof H) {
            set_error(RSG_ERR_IO, "rsg_read_internal: file is truncated in %s", path);
            return RSG_ERR_IO;
        }
        // the reference asserts these (src/io/io_internal.c:92-94)
        const char *bad = H.magic != kMagic                    ? "not a Rockstar binary file"
                          : H.particle_type != kParticleTypeFull ? "no full particle records"
                          : H.num_particles < 0                 ? "negative particle count"
                          : (int64_t)sb.st_size < (int64_t)sizeof H +
                                    H.num_particles * (int64_t)sizeof(rsg_particle)
                              ? "file is truncated"
                              : nullptr;
        if (bad) {
            set_error(RSG_ERR_IO, "rsg_read_internal: %s in %s", bad, path);
            return RSG_ERR_IO;
        }
        // read_binary_header_config: the header's floats into the doubles
        cfg->scale_now = H.scale;
        cfg->om = H.Om;
        cfg->ol = H.Ol;
        cfg->h0 = H.h0;
        cfg->box_size = H.box_size;
        cfg->particle_mass = H.particle_mass;
        const int64_t n = H.num_particles;
        *num_p = n;
        if (!want) return 0;  // the count alone
        if (n > max_p) {
            set_error(RSG_ERR_ARGS, "rsg_read_internal: %lld particles for %lld places",
                      (long long)n, (long long)max_p);
            return RSG_ERR_ARGS;
        }
        const size_t bytes = sizeof(rsg_particle) * (size_t)n;
        if (out_host)
            read_file_parallel(F.fd, sizeof H, out_host, bytes, path);
        else
            stage_h2d({{F.fd, (int64_t)sizeof H, nullptr, out_dev, bytes}}, path);
        return 0;
    } catch (Failure &) {
        return error_code();
    }
}

}  // namespace
}  // namespace rsg

using namespace rsg;

extern "C" int rsg_read_internal(const char *path, struct rsg_config *cfg, struct rsg_particle *p,
                                 int64_t max_p, int64_t *num_p) {
    return read_core(path, cfg, p, nullptr, max_p, num_p);
}

extern "C" int rsg_read_internal_device(const char *path, struct rsg_config *cfg,
                                        struct rsg_particle *d_p, int64_t max_p, int64_t *num_p) {
    return read_core(path, cfg, nullptr, d_p, max_p, num_p);
}

extern "C" int rsg_write_internal(const char *path, const struct rsg_particle *p, int64_t num_p,
                                  int64_t snap, int64_t chunk, const struct rsg_config *cfg) {
    if (!path || !cfg || num_p < 0 || (num_p && !p)) {
        set_error(RSG_ERR_ARGS, "rsg_write_internal: bad arguments");
        return RSG_ERR_ARGS;
    }
    BinHeader H;
    fill_header(H, snap, chunk, *cfg);
    H.num_particles = num_p;
    H.particle_type = kParticleTypeFull;
    FILE *o = fopen(path, "wb");
    if (!o) {
        set_error(RSG_ERR_IO, "rsg_write_internal: cannot open %s", path);
        return RSG_ERR_IO;
    }
    bool ok = fwrite(&H, sizeof H, 1, o) == 1;
    if (ok && num_p)
        ok = fwrite(p, sizeof(rsg_particle), (size_t)num_p, o) == (size_t)num_p;
    ok = (fclose(o) == 0) && ok;
    if (!ok) {
        set_error(RSG_ERR_IO, "rsg_write_internal: write to %s failed", path);
        return RSG_ERR_IO;
    }
    return 0;
}
