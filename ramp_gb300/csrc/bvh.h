#ifndef RAMP_BVH_H
#define RAMP_BVH_H
#include <cstdint>
#include <vector>

/* Build the GMesh hierarchy over float32 triangles pts[n_tri*9].
 * nodes: 16 floats per inner node, tris: 12 floats per triangle (mesh.cuh). */
int ramp_bvh_build(const float* pts, int64_t n_tri, std::vector<float>& nodes,
                   std::vector<float>& tris);

#endif
