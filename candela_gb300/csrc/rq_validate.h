// Host-side validation of uploaded scene buffers.  Every index a kernel can follow — child links,
// escape links, leaf triangle ranges, triangle vertex indices, entity node ranges — is checked
// once here, so the traversal kernels need no per-access bounds checks and never read out of
// bounds, whatever the caller passes.
#pragma once
#include <cstdint>
#include <string>

#include "../../include/rq.h"

namespace rq {

bool validate_scene(int32_t layout, const rq_vertex* verts, int64_t n_verts, const rq_triangle* tris,
                    int64_t n_tris, const void* nodes, int64_t n_nodes, const rq_entity* ents,
                    int32_t n_ents, std::string& why);

bool validate_entities(int32_t layout, const float* nodes, int64_t n_nodes, int64_t n_tris,
                       const rq_entity* ents, int32_t n_ents, std::string& why);

}  // namespace rq
