// mc_group.h — GroupTriangles (model3d/bvh.go:118-217) on the device, for
// SaveGroupedSTL (model3d/mesh.go:724-742).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mcgpu {

// Grow-only device buffers of the grouping; owned by a context.
struct GroupScratch;
GroupScratch* group_scratch_new();
void group_scratch_free(GroupScratch* g);

// The GroupTriangles permutation of T triangles (vertex-index triples into
// verts, float64 x y z; with tris null, triangle t is vertices 3t..3t+2):
// order[i] = the triangle placed i-th.  Each midpoint
// sort is stable, so ties keep the input order.  Runs on `stream`, waiting
// for it to pick the sort passes and at the end; *internal_error is set when
// a kernel's own consistency check failed (order is then not valid).
cudaError_t group_triangles_device(GroupScratch* g, const double* verts, const int32_t* tris, long long T,
                                   int32_t* order, cudaStream_t stream, int sm_count, bool* internal_error);

}  // namespace mcgpu
