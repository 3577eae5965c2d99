// mc_lower.h — host-side lowering of the mc_node serialisation into the
// device program layout of mc_internal.h.
#pragma once

#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/mcgpu.h"
#include "mc_internal.h"

namespace mcgpu {

struct LowerError : std::runtime_error {
    mc_status status;
    LowerError(mc_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

// Allocator whose default construction leaves elements uninitialised: the
// large arrays of a lowering are sized once and every element is then
// written by host threads, so the serial zero fill (and first touch of every
// page on one thread) is skipped.  Construction from a value is as usual.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept {
        ::new ((void*)p) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new ((void*)p) U(std::forward<A>(a)...);
    }
};
template <class T>
using bulk_vector = std::vector<T, NoInitAlloc<T>>;

// Host copy of a lowered solid; uploaded once by mc_solid_create.
struct HostProgram {
    std::vector<uint32_t> ops, ops_allfalse;
    int n_ops_allfalse = FOLD_FALSE;
    int fold_cap = 0;
    std::vector<int32_t> leaf_kind;
    std::vector<double> leaf_d;
    std::vector<float> leaf_f;
    std::vector<double> cull;
    std::vector<float> cull_f;
    std::vector<XBoxD> xbox;
    std::vector<XStepD> xstep;
    std::vector<TreeD> trees;
    bulk_vector<BvhNodeD> nodes;
    bulk_vector<BvhNodeF> nodes_f;
    std::vector<int32_t> tri_parent;
    bulk_vector<int32_t> cell_start;
    bulk_vector<RayEnt> ents;
    bulk_vector<TriD> tris;
    bulk_vector<TriF> tris_f;
    std::vector<MetaD> metas;
    std::vector<MetaF> metas_f;
    std::vector<BallD> balls;
    std::vector<BallF> balls_f;
    double root_min[3] = {0, 0, 0}, root_max[3] = {0, 0, 0};
    int max_stack = 0, max_xdepth = 0;
    bool has_collider = false;
    bool has_transform = false;
};

// Throws LowerError.
void lower_scene(const mc_node* nodes, size_t n_nodes, const mc_tri_set* sets, size_t n_sets,
                 HostProgram* out);

// Apply records of JoinedTransform(steps) (MC_XF_* records), or of its
// Inverse() when inverse is set; throws LowerError on a bad step kind.
std::vector<XStepD> transform_steps(const mc_node* steps, size_t n, bool inverse);

// math.Pow(x, y) for integer y, 0 < |y| < 2^20, x > 0 finite (Go math/pow.go).
double go_pow_int(double x, long y);

// newSquareSpacer for one axis; MC_OK or MC_ERR_GRID.
int spacer_axis(double lo, double hi, double delta, std::vector<double>* out, int64_t limit);

// LookupEdgePoint of every grid value (out[2k]) and edge midpoint (out[2k+1])
// of one spacer axis; delta = Xs[1] - Xs[0].  Codes: idx, -1 (not on an edge
// along this axis), -2 (index out of range).  out holds 2 * vals.size().
void edge_lookup_table(const std::vector<double>& vals, double delta, int32_t* out);

// mcLookupTable; 0 when all 256 cases are covered without conflicts.
int build_case_table(uint8_t counts[256], uint8_t tris[256][5][6]);

}  // namespace mcgpu
