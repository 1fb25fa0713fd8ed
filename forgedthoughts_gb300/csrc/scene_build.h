// Host-side construction of the GPU scene image: device node table, hard-union
// leaves, the leaf BVH, generic leaf programs and the culled union_round-tree
// structures.  Pure C++ (no CUDA) so it is shared by the renderer and the
// structure tests.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "forgedthoughts_gb300.h"
#include "ft_layout.h"

namespace ftgpu {

struct HostNode {  // mirrors ftd::DevNode (128 bytes)
  int32_t kind, a, b, program;
  uint32_t object_id, material_id;
  int32_t ival, has_rot;
  float c[3];
  float sz, cz, sy, cy, sx, cx;
  float f[6];
  float bmin[3], bmax[3];
  float pad[3];
};
static_assert(sizeof(HostNode) == 128, "HostNode layout");

struct HostLeaf {
  float bmin[3], bmax[3];
  int32_t kind;
  int32_t node;
  int32_t first;
  int32_t count;
};

struct HostBvhNode {  // leaf BVH in the reference's build order (R:693-732)
  float bmin[3], bmax[3];
  int32_t lhs, rhs, leaf, pad;
};

struct HostUrTree {
  float r;
  int32_t n_prims;
  int32_t prim_first;   // into ur_prims (in-order position -> node index)
  int32_t bvh_root;     // into ur_bvh
  int32_t inner_root;   // into ur_inner
  int32_t depth;
  int32_t fallback_first, fallback_count;  // generic program of the whole tree
  // Candidate grid: cell c lists every primitive that can be the nearest or
  // lie within r of some point of c.  dims[0] == 0 disables the grid.
  float gmin[3];
  float cell, inv_cell;
  int32_t dims[3];
  int32_t cell_first;  // into ur_cell_offsets (dims product + 1 entries)
  int32_t pad;
  // Outer grid: coarser cells over a box around the first grid, for points
  // outside it (there every primitive is at least 2r away, so a cell lists
  // the primitives that can be the nearest).  odims[0] == 0: none.
  float ogmin[3];
  float ocell, oinv_cell;
  int32_t odims[3];
  int32_t ocell_first;
  int32_t opad;
};

struct HostUrBvh {
  float bmin[3], bmax[3];
  int32_t left, right;
  int32_t prim_begin, prim_count;  // into ur_bvh_prims (in-order positions)
};

struct HostUrInner {
  int32_t child[2];  // >= 0: ur_inner index; < 0: -(position + 1) of a primitive
  int32_t lo, hi;    // in-order primitive range covered (relative to the tree)
};

struct SceneImage {
  std::vector<HostNode> nodes;
  std::vector<HostLeaf> leaves;
  std::vector<HostBvhNode> bvh;
  int32_t bvh_root = -1;
  std::vector<uint32_t> gops;
  std::vector<HostUrTree> urtrees;
  std::vector<HostUrBvh> ur_bvh;
  std::vector<int32_t> ur_bvh_prims;
  std::vector<int32_t> ur_prims;
  std::vector<HostUrInner> ur_inner;
  std::vector<uint32_t> ur_cell_offsets;  // per grid cell: begin into ur_cell_prims
  std::vector<int32_t> ur_cell_prims;     // in-order primitive positions
  // per ur_cell_prims entry: a lower bound of the distance from any point of
  // the cell to the primitive's box (the lists are sorted by it)
  std::vector<float> ur_cell_gaps;
  // per ur_cell_prims entry: the primitive's node index (ur_prims of it), so
  // the candidate walk loads it beside the position instead of after it
  std::vector<int32_t> ur_cell_nodes;
  // parent links of the union_round trees, (parent ur_inner index << 1) |
  // side, -1 at the root: per ur_inner node and per primitive position
  std::vector<int32_t> ur_inner_up;
  std::vector<int32_t> ur_prim_up;
  // per ur_inner node: 1 when its primitives use more than one material model
  // (blend_materials then yields a Blend whatever the weights)
  std::vector<int32_t> ur_inner_blend;
  std::vector<int32_t> node_op_begin, node_op_end;  // postfix op range of each node's subtree
  // per object id: the primitive or Custom node carrying it (its transform is
  // the object's, object_transforms R:485-555), -1 for none
  std::vector<int32_t> obj_node;
  std::vector<ft_material> materials;
  std::vector<ft_light> lights;
  int32_t environment_program = -1;
  std::vector<ft_program> programs;
  std::vector<ft_instr> instrs;
  float scene_min[3], scene_max[3];
  float scene_center[3];
  ft_camera camera;
  int32_t has_camera = 0;
  int32_t max_value_stack = 0, max_point_stack = 0;
};

// Build the image; returns false with `error` set on an invalid description.
bool build_scene_image(const ft_scene_desc& desc, SceneImage* out, std::string* error);

// Camera basis (R:6263-6286, render_api.rs:132-144) in f32.
struct CameraBasis {
  float origin[3], forward[3], right[3], up[3];
  float tan_fov;
};
CameraBasis resolve_camera(const SceneImage& img, const ft_render_options& opt);
// Basis of a camera at `org` looking at `tgt` (up (0, 1, 0)).
CameraBasis camera_basis(const float org[3], const float tgt[3], float fov);

}  // namespace ftgpu
