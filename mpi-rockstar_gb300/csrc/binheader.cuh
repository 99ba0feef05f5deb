// The reference's 256-byte binary file header (struct binary_output_header,
// src/io/io_internal.h:15-27), shared by the halo catalogue
// (halos_<snap>.<chunk>.bin) and the internal particle format
// (halos_<snap>.<chunk>.rbin).
#pragma once
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "rockstar_gb300.h"

namespace rsg {

using BinHeader = rsg_binary_header;
static_assert(sizeof(BinHeader) == 256, "binary header is 256 bytes");

constexpr uint64_t kMagic = 0xfadedacec0c0d0d0ull;  // ROCKSTAR_MAGIC
constexpr int32_t kFormatRevision = 2;              // HALO_FORMAT_REVISION, src/halo.h:4
constexpr const char *kVersion = "1.0.0RC";         // ROCKSTAR_VERSION, src/version.h:4
// OUTPUT_NFW_CHI2 (1) | OUTPUT_INERTIA_TENSOR (4): the build flags the halo
// layout follows (src/io/io_internal.c:30-40)
constexpr int32_t kAddFlag = 1 | 4;
constexpr int64_t kParticleTypeIds = 1;   // PARTICLE_TYPE_IDS
constexpr int64_t kParticleTypeFull = 2;  // PARTICLE_TYPE_FULL

// fill_binary_header (src/io/io_internal.c:16-41) on a zeroed header: the
// configuration's doubles stored as floats
inline void fill_header(BinHeader &H, int64_t snap, int64_t chunk, const rsg_config &c) {
    memset(&H, 0, sizeof H);
    H.magic = kMagic;
    H.snap = snap;
    H.chunk = chunk;
    H.scale = (float)c.scale_now;
    H.Om = (float)c.om;
    H.Ol = (float)c.ol;
    H.h0 = (float)c.h0;
    H.box_size = (float)c.box_size;
    H.particle_mass = (float)c.particle_mass;
    snprintf(H.rockstar_version, sizeof H.rockstar_version, "%s", kVersion);
    H.format_revision = kFormatRevision;
    H.add_flag = kAddFlag;
}

}  // namespace rsg
