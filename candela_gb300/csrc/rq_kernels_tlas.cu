// The ray-query kernels and launchers for scenes with a top level over their entities
// (rq_tlas.cuh): the same kernels as rq_kernels.cu, compiled with the entity cursor.
#include "rq_kernels.cuh"

namespace rq {

template cudaError_t launch_closest_t<true>(const SceneView&, const QueryConfig&, const rq_ray*, int64_t,
                                            rq_hit*, unsigned long long*, cudaStream_t);
template cudaError_t launch_anyhit_t<true>(const SceneView&, const QueryConfig&, const rq_ray*, int64_t,
                                           uint8_t*, unsigned long long*, cudaStream_t);

}  // namespace rq
