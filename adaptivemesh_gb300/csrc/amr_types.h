// amr_types.h -- host/device plain data shared by the kernels, the C ABI and the octree.
#pragma once

#include <cstdint>

#include "amr_gb300.h"

namespace amr {

constexpr uint32_t kDepthLimit = 8;           // AMR.h:9 (4-bit depth in domain_boundary)
constexpr uint32_t kPathMask = 134217727u;    // 27-bit Morton path of octree_abs_pos (AMR.h:22)

// Per-configuration scale factors, computed on the host in single precision exactly as the
// reference's constexprs and kernels compute them (AMR.h:16-17, 1176, 1214-1215, 1263).
struct Geo {
    float inv_dx[kDepthLimit + 1];    // 2^depth / outer_dx
    float inv_dx2[kDepthLimit + 1];   // inv_dx * inv_dx (rounded)
    float outer_dx;                   // outer_size / size_domain
    float outer_dt;                   // outer_dx * 0.4 (CFL 0.4)
};

inline Geo make_geo(const amr_config& c) {
    Geo g;
    volatile float osz = c.outer_size;   // keep the host compiler from folding in higher precision
    g.outer_dx = osz / (float)c.size_domain;
    g.outer_dt = g.outer_dx * .4f;
    for (uint32_t d = 0; d <= kDepthLimit; d++) {
        g.inv_dx[d] = (float)(1u << d) / g.outer_dx;
        g.inv_dx2[d] = g.inv_dx[d] * g.inv_dx[d];
    }
    return g;
}

}  // namespace amr
