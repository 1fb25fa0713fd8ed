// Host-side construction of the GPU scene image (see scene_build.h).
//
// Leaves are the operands of hard unions, collected as collect_accel_leaves
// does (R:659-670, R = crates/forgedthoughts/src/renderer.rs); the leaf BVH
// is built exactly as build_bvh (R:693-732): median split of leaf-AABB
// centroids along the longest axis with a stable sort, so a GPU traversal in
// the reference's order (R:743-786) visits leaves in the same sequence.
#include "scene_build.h"

#include "common.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <numeric>
#include <string>
#include <atomic>
#include <exception>
#include <mutex>
#include <system_error>
#include <thread>

namespace ftgpu {
namespace {

// Edge, in cells, of the blocks the candidate grid is built in.
constexpr int kGridBlock = 4;
// Candidate-list entries of all union_round grids of a scene (8 bytes each on
// the device); trees past it evaluate through their BVH.
constexpr uint64_t kMaxGridEntries = uint64_t(1) << 26;

struct Box {
  float mn[3], mx[3];
};

Box box_union(const Box& a, const Box& b) {
  Box o;
  for (int k = 0; k < 3; ++k) {
    o.mn[k] = std::min(a.mn[k], b.mn[k]);
    o.mx[k] = std::max(a.mx[k], b.mx[k]);
  }
  return o;
}

bool is_prim(int k) { return k >= FT_NODE_SPHERE && k <= FT_NODE_EXTRUDE_POLYGON; }
bool is_binary(int k) { return k >= FT_NODE_UNION && k <= FT_NODE_TONGUE; }
bool is_unary(int k) {
  return k == FT_NODE_DOMAIN || k == FT_NODE_DISTANCE_POST || k == FT_NODE_NOISE || k == FT_NODE_SLICE ||
         k == FT_NODE_SMOOTH;
}

float deg_to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

class Builder {
 public:
  Builder(const ft_scene_desc& d, SceneImage* img, std::string* err) : d_(d), img_(img), err_(err) {}

  bool run() {
    if (!validate()) return false;
    convert_nodes();
    bounds_.assign(d_.n_nodes, Box{});
    have_bounds_.assign(d_.n_nodes, 0);
    for (uint32_t i = 0; i < d_.n_nodes; ++i) node_bounds(static_cast<int>(i));
    // Primitive nodes carry their culling box in bmin/bmax.
    for (uint32_t i = 0; i < d_.n_nodes; ++i) {
      if (is_prim(d_.nodes[i].kind) || d_.nodes[i].kind == FT_NODE_CUSTOM) {
        std::memcpy(img_->nodes[i].bmin, bounds_[i].mn, sizeof(float) * 3);
        std::memcpy(img_->nodes[i].bmax, bounds_[i].mx, sizeof(float) * 3);
      }
    }
    // Object id -> the node carrying its transform (the shading context's
    // local position of a hit, build_bsdf_context R:4403-4408).
    for (uint32_t i = 0; i < d_.n_nodes; ++i) {
      const ft_node& n = d_.nodes[i];
      if (!(is_prim(n.kind) || n.kind == FT_NODE_CUSTOM) || n.object_id >= (1u << 20)) continue;
      if (img_->obj_node.size() <= n.object_id) img_->obj_node.resize(n.object_id + 1, -1);
      if (img_->obj_node[n.object_id] < 0) img_->obj_node[n.object_id] = static_cast<int32_t>(i);
    }
    const Box& sb = bounds_[d_.root];
    std::memcpy(img_->scene_min, sb.mn, sizeof(sb.mn));
    std::memcpy(img_->scene_max, sb.mx, sizeof(sb.mx));
    std::memcpy(img_->scene_center, d_.scene_center, sizeof(d_.scene_center));
    img_->camera = d_.camera;
    img_->has_camera = d_.has_camera;
    img_->programs.assign(d_.programs, d_.programs + d_.n_programs);
    img_->instrs.assign(d_.instrs, d_.instrs + d_.n_instrs);
    img_->materials.assign(d_.materials, d_.materials + d_.n_materials);
    img_->lights.assign(d_.lights, d_.lights + d_.n_lights);
    img_->environment_program = d_.environment_program;
    if (img_->materials.empty()) {  // default_material (R:7937-7953)
      ft_material m;
      std::memset(&m, 0, sizeof(m));
      m.kind = FT_MAT_STANDARD;
      m.color_program = m.roughness_program = m.ior_program = m.thin_walled_program = -1;
      for (int32_t& h : m.hook_program) h = -1;
      m.color[0] = m.color[1] = m.color[2] = 0.8f;
      m.roughness = 0.5f;
      m.ior = 1.5f;
      m.specular = 0.5f;
      m.specular_weight = 1.0f;
      m.specular_color[0] = m.specular_color[1] = m.specular_color[2] = 1.0f;
      m.clearcoat_roughness = 0.1f;
      img_->materials.push_back(m);
    }
    img_->node_op_begin.assign(d_.n_nodes, -1);
    img_->node_op_end.assign(d_.n_nodes, -1);

    collect_leaves(d_.root);
    std::vector<size_t> idx(img_->leaves.size());
    std::iota(idx.begin(), idx.end(), 0);
    img_->bvh_root = build_bvh(idx);
    for (size_t li = 0; li < img_->leaves.size(); ++li)
      if (!classify(li)) return false;
    return true;
  }

 private:
  const ft_scene_desc& d_;
  SceneImage* img_;
  std::string* err_;
  std::vector<Box> bounds_;
  std::vector<char> have_bounds_;

  bool fail(const std::string& m) {
    *err_ = m;
    return false;
  }

  // Every index that a kernel dereferences is checked here, on the host.
  bool validate() {
    if (d_.abi_version != FT_ABI_VERSION) return fail("scene description has a different ABI version");
    if (d_.n_nodes == 0 || !d_.nodes) return fail("scene has no nodes");
    if (d_.root < 0 || static_cast<uint32_t>(d_.root) >= d_.n_nodes) return fail("scene root index out of range");
    for (uint32_t i = 0; i < d_.n_programs; ++i) {
      const ft_program& p = d_.programs[i];
      if (p.n_regs > FT_MAX_PROGRAM_REGS || p.n_params > p.n_regs || p.n_instr == 0)
        return fail("hook program " + std::to_string(i) + " has an invalid register/instruction count");
      if (static_cast<uint64_t>(p.first_instr) + p.n_instr > d_.n_instrs)
        return fail("hook program " + std::to_string(i) + " instruction range out of bounds");
      for (uint32_t k = 0; k < p.n_instr; ++k) {
        const ft_instr& in = d_.instrs[p.first_instr + k];
        if (in.op >= FT_OP_COUNT) return fail("hook program has an unknown opcode");
        if (in.dst >= p.n_regs || in.a >= p.n_regs || in.b >= p.n_regs || in.c >= p.n_regs)
          return fail("hook program register index out of range");
      }
      if (d_.instrs[p.first_instr + p.n_instr - 1].op != FT_OP_RET)
        return fail("hook program does not end with a return");
    }
    for (uint32_t i = 0; i < d_.n_nodes; ++i) {
      const ft_node& n = d_.nodes[i];
      if (n.kind < 0 || n.kind >= FT_NODE_KIND_COUNT) return fail("node " + std::to_string(i) + " has an unknown kind");
      auto child_ok = [&](int c) { return c >= 0 && static_cast<uint32_t>(c) < d_.n_nodes && c != static_cast<int>(i); };
      if (is_binary(n.kind) && (!child_ok(n.a) || !child_ok(n.b)))
        return fail("node " + std::to_string(i) + " has an invalid child index");
      if (is_unary(n.kind) && !child_ok(n.a)) return fail("node " + std::to_string(i) + " has an invalid base index");
      if (n.kind == FT_NODE_DOMAIN || n.kind == FT_NODE_DISTANCE_POST) {
        if (n.program < 0 || static_cast<uint32_t>(n.program) >= d_.n_programs)
          return fail("modifier node " + std::to_string(i) + " has an invalid program index");
        const ft_program& p = d_.programs[n.program];
        bool dom = n.kind == FT_NODE_DOMAIN;
        if (dom && (p.n_params != 1 || p.param_is_vec3 != 1u || !p.result_is_vec3))
          return fail("domain hook must map vec3 -> vec3");
        if (!dom && (p.n_params != 2 || p.param_is_vec3 != 2u || p.result_is_vec3))
          return fail("distance_post hook must map (f32, vec3) -> f32");
      }
      if (n.kind == FT_NODE_SLICE && (n.ival < 0 || n.ival > 2)) return fail("slice axis out of range");
      if (n.kind == FT_NODE_CUSTOM) {
        // distance(p) -> f32, domain(p) -> vec3, distance_post(d, p) -> f32
        auto prog_ok = [&](int32_t idx, uint32_t np, uint32_t vec_mask, bool vec_result, bool required) {
          if (idx < 0) return !required;
          if (static_cast<uint32_t>(idx) >= d_.n_programs) return false;
          const ft_program& p = d_.programs[idx];
          return p.n_params == np && p.param_is_vec3 == vec_mask && (p.result_is_vec3 != 0) == vec_result;
        };
        if (!prog_ok(n.program, 1, 1u, false, true) || !prog_ok(n.ival, 1, 1u, true, false) ||
            !prog_ok(n.reserved, 2, 2u, false, false))
          return fail("custom sdf node " + std::to_string(i) + " has an invalid program");
        if (!(n.f[0] > 0.0f && n.f[1] > 0.0f && n.f[2] > 0.0f))
          return fail("custom sdf node " + std::to_string(i) + " has invalid bounds");
      }
    }
    if (d_.environment_program >= 0) {
      if (static_cast<uint32_t>(d_.environment_program) >= d_.n_programs)
        return fail("environment program index out of range");
      const ft_program& p = d_.programs[d_.environment_program];
      if (p.n_params != 1 || p.param_is_vec3 != 1u || !p.result_is_vec3)
        return fail("environment color program must map vec3 -> vec3");
    }
    if (d_.n_lights && !d_.lights) return fail("lights pointer is null");
    if (d_.n_materials && !d_.materials) return fail("materials pointer is null");
    for (uint32_t i = 0; i < d_.n_lights; ++i) {
      if (d_.lights[i].kind < FT_LIGHT_POINT || d_.lights[i].kind > FT_LIGHT_SPHERE)
        return fail("light " + std::to_string(i) + " has an unknown kind");
      if (d_.lights[i].samples > 4096) return fail("light " + std::to_string(i) + " has too many samples");
    }
    for (uint32_t i = 0; i < d_.n_materials; ++i) {
      const ft_material& m = d_.materials[i];
      if (m.kind < FT_MAT_STANDARD || m.kind > FT_MAT_DIELECTRIC)
        return fail("material " + std::to_string(i) + " has an unknown kind");
      // Each hook slot: the program index, then its context (7 shading or 13
      // BSDF parameters) and result (0 number, 1 vec3, 2 either).
      struct Want {
        int32_t prog;
        bool bsdf;
        int result;
      };
      std::vector<Want> wants = {{m.color_program, false, 2}, {m.roughness_program, false, 0},
                                 {m.ior_program, false, 0}, {m.thin_walled_program, false, 0}};
      static const int kResult[FT_MATERIAL_HOOKS] = {2, 0, 0, 0, 0, 0, 2, 0, 0, 0, 0, 0, 1,  // properties, bump, normal
                                                     2, 0,                                  // eval, pdf
                                                     1, 2, 0, 0, 0, 0, 0, 0,                // sample fields
                                                     0, 2, 0};                              // medium fields
      for (int k = 0; k < FT_MATERIAL_HOOKS; ++k)
        wants.push_back({m.hook_program[k], k >= FT_HOOK_EVAL && k <= FT_HOOK_SAMPLE_NEXT_IOR, kResult[k]});
      for (int k = FT_MATERIAL_HOOKS; k < FT_MATERIAL_HOOK_SLOTS; ++k)
        if (m.hook_program[k] != -1) return fail("material " + std::to_string(i) + " uses a reserved hook slot");
      for (const Want& w : wants) {
        if (w.prog < 0) continue;
        if (static_cast<uint32_t>(w.prog) >= d_.n_programs)
          return fail("material " + std::to_string(i) + " has an invalid hook program index");
        const ft_program& p = d_.programs[w.prog];
        const uint32_t np = w.bsdf ? FT_BSDF_HOOK_PARAMS : FT_MATERIAL_HOOK_PARAMS;
        const uint32_t vec_mask = w.bsdf ? 0x18fu : 0xfu;
        if (p.n_params != np || p.param_is_vec3 != vec_mask || (w.result == 0 && p.result_is_vec3) ||
            (w.result == 1 && !p.result_is_vec3))
          return fail("material " + std::to_string(i) + " hook must map the " +
                      (w.bsdf ? "BSDF" : "shading") + " context to " +
                      (w.result == 0 ? "a number" : w.result == 1 ? "a vec3" : "a colour"));
      }
    }
    // The node graph must be a DAG reachable from the root (no cycles).
    std::vector<char> state(d_.n_nodes, 0);
    std::function<bool(int, int)> dfs = [&](int i, int depth) -> bool {
      if (depth > 100000) return false;
      if (state[i] == 1) return false;
      if (state[i] == 2) return true;
      state[i] = 1;
      const ft_node& n = d_.nodes[i];
      if ((is_binary(n.kind) || is_unary(n.kind)) && !dfs(n.a, depth + 1)) return false;
      if (is_binary(n.kind) && !dfs(n.b, depth + 1)) return false;
      state[i] = 2;
      return true;
    };
    if (!dfs(d_.root, 0)) return fail("scene node graph has a cycle or is too deep");
    return true;
  }

  void convert_nodes() {
    img_->nodes.resize(d_.n_nodes);
    for (uint32_t i = 0; i < d_.n_nodes; ++i) {
      const ft_node& s = d_.nodes[i];
      HostNode& n = img_->nodes[i];
      std::memset(&n, 0, sizeof(n));
      n.kind = s.kind;
      n.a = s.a;
      n.b = s.b;
      n.program = s.program;
      n.object_id = s.object_id;
      n.material_id = s.material_id;
      n.ival = s.ival;
      std::memcpy(n.c, s.center, sizeof(n.c));
      n.has_rot = (s.rot_deg[0] != 0.0f || s.rot_deg[1] != 0.0f || s.rot_deg[2] != 0.0f) ? 1 : 0;
      // to_local rotates by the negated angles (R:6216-6222).
      float rz = deg_to_rad(-s.rot_deg[2]), ry = deg_to_rad(-s.rot_deg[1]), rx = deg_to_rad(-s.rot_deg[0]);
      n.sz = std::sin(rz); n.cz = std::cos(rz);
      n.sy = std::sin(ry); n.cy = std::cos(ry);
      n.sx = std::sin(rx); n.cx = std::cos(rx);
      std::memcpy(n.f, s.f, sizeof(n.f));
      std::memcpy(n.bmin, s.bounds_min, sizeof(n.bmin));
      std::memcpy(n.bmax, s.bounds_max, sizeof(n.bmax));
      if (s.kind == FT_NODE_CUSTOM) {  // a leaf: program distance, ival domain, b distance_post
        n.a = -1;
        n.b = s.reserved;
      }
    }
  }

  // sdf_bounds (R:5242-5386) in f32.
  const Box& node_bounds(int i) {
    if (have_bounds_[i]) return bounds_[i];
    const ft_node& n = d_.nodes[i];
    Box b{};
    auto cube = [&](float r) {
      for (int k = 0; k < 3; ++k) {
        b.mn[k] = n.center[k] - r;
        b.mx[k] = n.center[k] + r;
      }
    };
    switch (n.kind) {
      case FT_NODE_SPHERE: cube(n.f[0]); break;
      case FT_NODE_BOX: cube(std::sqrt(n.f[0] * n.f[0] + n.f[1] * n.f[1] + n.f[2] * n.f[2])); break;
      case FT_NODE_CYLINDER:
      case FT_NODE_EXTRUDE_POLYGON: cube(std::sqrt(n.f[0] * n.f[0] + n.f[1] * n.f[1])); break;
      case FT_NODE_TORUS: cube(n.f[0] + n.f[1]); break;
      case FT_NODE_DOMAIN:
      case FT_NODE_DISTANCE_POST:
      case FT_NODE_NOISE:
      case FT_NODE_CUSTOM:
        std::memcpy(b.mn, n.bounds_min, sizeof(b.mn));
        std::memcpy(b.mx, n.bounds_max, sizeof(b.mx));
        break;
      case FT_NODE_SUBTRACT: b = node_bounds(n.a); break;
      case FT_NODE_SLICE: {
        b = node_bounds(n.a);
        int ax = n.ival;
        b.mn[ax] = std::max(b.mn[ax], n.f[0]);
        b.mx[ax] = std::min(b.mx[ax], n.f[1]);
        if (b.mx[ax] < b.mn[ax]) b.mx[ax] = b.mn[ax];
        break;
      }
      case FT_NODE_SMOOTH: {
        b = node_bounds(n.a);
        float e = n.f[0] * 0.1f;
        for (int k = 0; k < 3; ++k) {
          b.mn[k] -= e;
          b.mx[k] += e;
        }
        break;
      }
      default: b = box_union(node_bounds(n.a), node_bounds(n.b)); break;
    }
    bounds_[i] = b;
    have_bounds_[i] = 1;
    return bounds_[i];
  }

  void collect_leaves(int i) {
    const ft_node& n = d_.nodes[i];
    if (n.kind == FT_NODE_UNION) {
      collect_leaves(n.a);
      collect_leaves(n.b);
      return;
    }
    HostLeaf l;
    std::memset(&l, 0, sizeof(l));
    const Box& b = bounds_[i];
    std::memcpy(l.bmin, b.mn, sizeof(b.mn));
    std::memcpy(l.bmax, b.mx, sizeof(b.mx));
    l.node = i;
    img_->leaves.push_back(l);
  }

  int build_bvh(const std::vector<size_t>& indices) {
    if (indices.empty()) return -1;
    auto& leaves = img_->leaves;
    HostBvhNode node;
    std::memset(&node, 0, sizeof(node));
    node.lhs = node.rhs = node.leaf = -1;
    if (indices.size() == 1) {
      std::memcpy(node.bmin, leaves[indices[0]].bmin, sizeof(node.bmin));
      std::memcpy(node.bmax, leaves[indices[0]].bmax, sizeof(node.bmax));
      node.leaf = static_cast<int32_t>(indices[0]);
      img_->bvh.push_back(node);
      return static_cast<int>(img_->bvh.size()) - 1;
    }
    Box b;
    std::memcpy(b.mn, leaves[indices[0]].bmin, sizeof(b.mn));
    std::memcpy(b.mx, leaves[indices[0]].bmax, sizeof(b.mx));
    for (size_t k = 1; k < indices.size(); ++k) {
      Box o;
      std::memcpy(o.mn, leaves[indices[k]].bmin, sizeof(o.mn));
      std::memcpy(o.mx, leaves[indices[k]].bmax, sizeof(o.mx));
      b = box_union(b, o);
    }
    float ex = b.mx[0] - b.mn[0], ey = b.mx[1] - b.mn[1], ez = b.mx[2] - b.mn[2];
    int axis = (ex >= ey && ex >= ez) ? 0 : (ey >= ez ? 1 : 2);
    auto centroid = [&](size_t li) { return (leaves[li].bmin[axis] + leaves[li].bmax[axis]) * 0.5f; };
    std::vector<size_t> sorted = indices;
    std::stable_sort(sorted.begin(), sorted.end(), [&](size_t x, size_t y) { return centroid(x) < centroid(y); });
    size_t mid = sorted.size() / 2;
    int l = build_bvh(std::vector<size_t>(sorted.begin(), sorted.begin() + mid));
    int r = build_bvh(std::vector<size_t>(sorted.begin() + mid, sorted.end()));
    std::memcpy(node.bmin, b.mn, sizeof(node.bmin));
    std::memcpy(node.bmax, b.mx, sizeof(node.bmax));
    node.lhs = l;
    node.rhs = r;
    img_->bvh.push_back(node);
    return static_cast<int>(img_->bvh.size()) - 1;
  }

  // Postfix program over a leaf's node tree; tracks stack depths.
  // Postfix ops of every subtree are contiguous: record each node's range so a
  // shading pass can re-evaluate any subtree at arbitrary points.
  bool emit_generic(int i, int vdepth, int pdepth, int* vmax, int* pmax) {
    int32_t begin = static_cast<int32_t>(img_->gops.size());
    bool ok = emit_generic_ops(i, vdepth, pdepth, vmax, pmax);
    img_->node_op_begin[i] = begin;
    img_->node_op_end[i] = static_cast<int32_t>(img_->gops.size());
    return ok;
  }

  bool emit_generic_ops(int i, int vdepth, int pdepth, int* vmax, int* pmax) {
    const ft_node& n = d_.nodes[i];
    auto op = [&](uint32_t code) { img_->gops.push_back((code << kGOpShift) | static_cast<uint32_t>(i)); };
    *pmax = std::max(*pmax, pdepth);
    if (static_cast<uint32_t>(i) > kGNodeMask) return fail("scene has too many nodes for the generic evaluator");
    if (is_prim(n.kind)) {
      op(kGPrim);
      *vmax = std::max(*vmax, vdepth + 1);
      return true;
    }
    if (n.kind == FT_NODE_CUSTOM) {
      op(kGCustom);
      *vmax = std::max(*vmax, vdepth + 1);
      return true;
    }
    switch (n.kind) {
      case FT_NODE_DOMAIN:
        op(kGDomainPush);
        if (!emit_generic(n.a, vdepth, pdepth + 1, vmax, pmax)) return false;
        op(kGPop);
        return true;
      case FT_NODE_DISTANCE_POST:
        op(kGLocalPush);
        if (!emit_generic(n.a, vdepth, pdepth + 1, vmax, pmax)) return false;
        op(kGPostPop);
        return true;
      case FT_NODE_NOISE:
        op(kGLocalPush);
        if (!emit_generic(n.a, vdepth, pdepth + 1, vmax, pmax)) return false;
        op(kGNoisePop);
        return true;
      case FT_NODE_SLICE:
        if (!emit_generic(n.a, vdepth, pdepth, vmax, pmax)) return false;
        op(kGSlice);
        return true;
      case FT_NODE_SMOOTH:
        if (!emit_generic(n.a, vdepth, pdepth, vmax, pmax)) return false;
        op(kGSmooth);
        return true;
      default:
        if (!emit_generic(n.a, vdepth, pdepth, vmax, pmax)) return false;
        if (!emit_generic(n.b, vdepth + 1, pdepth, vmax, pmax)) return false;
        op(kGBinary);
        return true;
    }
  }

  bool emit_program(int root, int32_t* first, int32_t* count) {
    *first = static_cast<int32_t>(img_->gops.size());
    int vmax = 0, pmax = 0;
    if (!emit_generic(root, 0, 0, &vmax, &pmax)) return false;
    *count = static_cast<int32_t>(img_->gops.size()) - *first;
    if (vmax > kMaxGenericValueStack || pmax >= kMaxGenericPointStack)
      return fail("scene leaf nests operators deeper than the generic evaluator supports (" +
                  std::to_string(vmax) + " values, " + std::to_string(pmax) + " points)");
    img_->max_value_stack = std::max(img_->max_value_stack, vmax);
    img_->max_point_stack = std::max(img_->max_point_stack, pmax);
    return true;
  }

  static float processed_r(float r) { return std::max(std::fabs(r), 1.0e-6f); }

  // A leaf qualifies for the culled union_round path if every inner node is
  // union_round with one radius and every leaf is a plain primitive.
  bool is_urtree(int root, float* r, int* nprims, int* depth) {
    const ft_node& rn = d_.nodes[root];
    if (rn.kind != FT_NODE_UNION_ROUND) return false;
    *r = processed_r(rn.f[0]);
    *nprims = 0;
    *depth = 0;
    std::function<bool(int, int)> walk = [&](int i, int dep) -> bool {
      const ft_node& n = d_.nodes[i];
      *depth = std::max(*depth, dep);
      if (is_prim(n.kind)) {
        ++*nprims;
        // Extruded polygons evaluate a distance to an edge line, which can lie
        // below their box bound; such trees take the exact generic path.
        return n.kind != FT_NODE_EXTRUDE_POLYGON;
      }
      if (n.kind != FT_NODE_UNION_ROUND || processed_r(n.f[0]) != *r) return false;
      return walk(n.a, dep + 1) && walk(n.b, dep + 1);
    };
    return walk(root, 1) && *nprims >= 4 && *depth <= kMaxUrDepth;
  }

  int build_ur_bvh(std::vector<int32_t>& pos, size_t lo, size_t hi, int32_t prim_first) {
    HostUrBvh node;
    std::memset(&node, 0, sizeof(node));
    node.left = node.right = -1;
    Box b;
    bool first = true;
    for (size_t k = lo; k < hi; ++k) {
      const HostNode& pn = img_->nodes[img_->ur_prims[prim_first + pos[k]]];
      Box o;
      std::memcpy(o.mn, pn.bmin, sizeof(o.mn));
      std::memcpy(o.mx, pn.bmax, sizeof(o.mx));
      b = first ? o : box_union(b, o);
      first = false;
    }
    std::memcpy(node.bmin, b.mn, sizeof(node.bmin));
    std::memcpy(node.bmax, b.mx, sizeof(node.bmax));
    int self = static_cast<int>(img_->ur_bvh.size());
    img_->ur_bvh.push_back(node);
    if (hi - lo <= static_cast<size_t>(kUrBvhLeafSize)) {
      img_->ur_bvh[self].prim_begin = static_cast<int32_t>(img_->ur_bvh_prims.size());
      img_->ur_bvh[self].prim_count = static_cast<int32_t>(hi - lo);
      for (size_t k = lo; k < hi; ++k) img_->ur_bvh_prims.push_back(pos[k]);
      return self;
    }
    // Median split of primitive-box centroids along the longest centroid axis.
    float cmn[3] = {std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity(),
                    std::numeric_limits<float>::infinity()};
    float cmx[3] = {-cmn[0], -cmn[1], -cmn[2]};
    auto cen = [&](int32_t p, int ax) {
      const HostNode& pn = img_->nodes[img_->ur_prims[prim_first + p]];
      return (pn.bmin[ax] + pn.bmax[ax]) * 0.5f;
    };
    for (size_t k = lo; k < hi; ++k)
      for (int ax = 0; ax < 3; ++ax) {
        cmn[ax] = std::min(cmn[ax], cen(pos[k], ax));
        cmx[ax] = std::max(cmx[ax], cen(pos[k], ax));
      }
    int axis = 0;
    for (int ax = 1; ax < 3; ++ax)
      if (cmx[ax] - cmn[ax] > cmx[axis] - cmn[axis]) axis = ax;
    size_t mid = (lo + hi) / 2;
    std::nth_element(pos.begin() + lo, pos.begin() + mid, pos.begin() + hi,
                     [&](int32_t x, int32_t y) { return cen(x, axis) < cen(y, axis); });
    int l = build_ur_bvh(pos, lo, mid, prim_first);
    int r = build_ur_bvh(pos, mid, hi, prim_first);
    img_->ur_bvh[self].left = l;
    img_->ur_bvh[self].right = r;
    return self;
  }

  // material_for_id (R:6895-6900): out-of-range ids fall back to material 0.
  int material_kind(uint32_t id) const {
    if (img_->materials.empty()) return FT_MAT_STANDARD;
    return img_->materials[id < img_->materials.size() ? id : 0].kind;
  }

  // Radius of a ball around the primitive's centre that lies inside the solid
  // (its distance is at most |p - c| - radius everywhere), or a negative value
  // when the shape has no such ball and the loose bound |p - c| + R applies.
  float inscribed_radius(const HostNode& n) const {
    switch (n.kind) {
      case FT_NODE_SPHERE: return n.f[1] > 0.0f ? -1.0f : n.f[0];
      case FT_NODE_BOX: return n.f[4] > 0.0f ? -1.0f : std::min(n.f[0], std::min(n.f[1], n.f[2]));
      default: return -1.0f;
    }
  }

  // Candidate grid over the tree's primitives.  For a cell C and primitive i,
  //   lb(i, C) = distance between i's AABB and C  (<= d_i(p) for p in C, p
  //              outside the AABB; the only case where lb > 0)
  //   ub(i, C) = max_{p in C} |p - c_i| - rho_i  (>= d_i(p), rho_i the
  //              inscribed radius; + R_i for shapes without one)
  // and C lists {i : lb(i, C) < max(r, min_j ub(j, C))}.  A primitive left out
  // has d >= r at every point of C (so it is inert in every union_round it
  // feeds) and d >= the cell's nearest distance, so evaluating only the list
  // gives the tree's exact value.  Cells are padded by a thousandth of their
  // size against rounding in the device's cell lookup.
  void build_ur_grid(HostUrTree& t) {
    const int np = t.n_prims;
    GridPrims g;
    g.np = np;
    g.pb.resize(np);
    g.cx.resize(np); g.cy.resize(np); g.cz.resize(np); g.rho.resize(np); g.rad.resize(np);
    std::vector<Box>& pb = g.pb;
    std::vector<float>&cx = g.cx, &cy = g.cy, &cz = g.cz, &rho = g.rho, &rad = g.rad;
    Box all{};
    for (int k = 0; k < np; ++k) {
      const HostNode& n = img_->nodes[img_->ur_prims[t.prim_first + k]];
      std::memcpy(pb[k].mn, n.bmin, sizeof(pb[k].mn));
      std::memcpy(pb[k].mx, n.bmax, sizeof(pb[k].mx));
      all = k ? box_union(all, pb[k]) : pb[k];
      cx[k] = n.c[0];
      cy[k] = n.c[1];
      cz[k] = n.c[2];
      rho[k] = inscribed_radius(n);
      rad[k] = 0.5f * (n.bmax[0] - n.bmin[0]);
    }
    for (int a = 0; a < 3; ++a) {
      all.mn[a] -= 2.0f * t.r;
      all.mx[a] += 2.0f * t.r;
    }
    double ext[3] = {double(all.mx[0]) - all.mn[0], double(all.mx[1]) - all.mn[1], double(all.mx[2]) - all.mn[2]};
    double target = std::min(262144.0, std::max(4096.0, 256.0 * np));
    double cell = std::cbrt(ext[0] * ext[1] * ext[2] / target);
    if (!(cell > 0.0) || !std::isfinite(cell)) return;
    int dims[3];
    for (int a = 0; a < 3; ++a) dims[a] = std::max(1, static_cast<int>(std::ceil(ext[a] / cell)));
    if (static_cast<int64_t>(dims[0]) * dims[1] * dims[2] > 2 * 262144) return;
    int32_t first = 0;
    if (!build_cells(t, g, all.mn, static_cast<float>(cell), dims, &first)) return;
    t.cell = static_cast<float>(cell);
    t.inv_cell = 1.0f / t.cell;
    std::memcpy(t.gmin, all.mn, sizeof(t.gmin));
    std::memcpy(t.dims, dims, sizeof(dims));
    t.cell_first = first;
    // The outer grid: the first grid's box widened by half its largest extent
    // on every side, in coarser cells.  Points there are outside the first
    // grid, hence at least 2r from every primitive box: each cell lists the
    // primitives that can be the nearest, sorted by gap, as above (a walk of
    // the tree's BVH from such points tests about six times as many boxes).
    // Points outside both grids take the tree BVH.
    const double widen = 0.5 * std::max({ext[0], ext[1], ext[2]});
    Box outer = all;
    for (int a = 0; a < 3; ++a) {
      outer.mn[a] = static_cast<float>(double(all.mn[a]) - widen);
      outer.mx[a] = static_cast<float>(double(all.mx[a]) + widen);
    }
    double oext[3] = {double(outer.mx[0]) - outer.mn[0], double(outer.mx[1]) - outer.mn[1],
                      double(outer.mx[2]) - outer.mn[2]};
    double otarget = std::min(double(1 << 19), std::max(32768.0, 256.0 * np));
    double ocell = std::cbrt(oext[0] * oext[1] * oext[2] / otarget);
    if (!(ocell > 0.0) || !std::isfinite(ocell)) return;
    int odims[3];
    for (int a = 0; a < 3; ++a) odims[a] = std::max(1, static_cast<int>(std::ceil(oext[a] / ocell)));
    if (static_cast<int64_t>(odims[0]) * odims[1] * odims[2] > 2 * (1 << 19)) return;
    if (!build_cells(t, g, outer.mn, static_cast<float>(ocell), odims, &first)) return;
    t.ocell = static_cast<float>(ocell);
    t.oinv_cell = 1.0f / t.ocell;
    std::memcpy(t.ogmin, outer.mn, sizeof(t.ogmin));
    std::memcpy(t.odims, odims, sizeof(odims));
    t.ocell_first = first;
  }

  // Primitive data of one union_round tree for its candidate grids.
  struct GridPrims {
    int np = 0;
    std::vector<Box> pb;
    std::vector<float> cx, cy, cz, rho, rad;
  };

  // Candidate lists of the dims[0] x dims[1] x dims[2] cells of size `cell`
  // from `gmin`: each cell lists every primitive that can be the nearest or
  // lie within r of one of its points, sorted by a lower bound of its box gap.
  // Appended to the image's cell arrays, the first cell's offset index in
  // *cell_first; false, with nothing appended, when the image's entry cap
  // would be passed.
  bool build_cells(const HostUrTree& t, const GridPrims& g, const float gmin[3], float cell, const int dims[3],
                   int32_t* cell_first) {
    const int np = g.np;
    const std::vector<Box>& pb = g.pb;
    const std::vector<float>&cx = g.cx, &cy = g.cy, &cz = g.cz, &rho = g.rho, &rad = g.rad;
    const double pad = double(cell) * 1.0e-3;
    const double half = 0.5 * double(cell);
    // Absolute rounding allowance of the block bounds below: far above the
    // error of a few double operations on the scene's coordinates.
    double scale = 0.0;
    for (int a = 0; a < 3; ++a)
      scale = std::max({scale, std::fabs(double(gmin[a])), std::fabs(double(gmin[a]) + double(dims[a]) * double(cell))});
    const double slack = 1e-9 * (1.0 + scale);
    // Padded extent of the cells [i0, i1) along axis a (one cell: i1 = i0 + 1).
    auto extent = [&](int a, int i0, int i1, double* lo, double* hi) {
      *lo = double(gmin[a]) + double(i0) * double(cell) - pad;
      *hi = double(gmin[a]) + double(i1) * double(cell) + pad;
    };
    // Cells are taken in blocks of kGridBlock^3.  For a block, T bounds every
    // cell's min_j ub(j, C) from above (the smallest ub of any one primitive
    // over the whole block), and two subsets of the primitives are kept:
    //   near:  lb of ub(i, C) over the block's cells < T, with
    //          ub(i, C) >= |(d_a + cell/2)_a| - rho_i, d_a the distance from
    //          c_i to the block along axis a (a cell's farthest face is at
    //          least that far);
    //   cands: box gap to the block < the largest threshold T allows.
    // A primitive outside `near` cannot give a cell's minimum and one outside
    // `cands` cannot pass a cell's threshold, so each cell's minimum and list,
    // computed over the subsets with the same expressions, are those of all
    // primitives.  The bounds carry `slack` against rounding.
    const int blk = kGridBlock;
    const int nbx = (dims[0] + blk - 1) / blk, nby = (dims[1] + blk - 1) / blk, nbz = (dims[2] + blk - 1) / blk;
    const size_t nrows = static_cast<size_t>(dims[1]) * dims[2];
    std::vector<std::vector<uint32_t>> row_offsets(nrows);
    std::vector<std::vector<int32_t>> row_prims(nrows);
    std::vector<std::vector<float>> row_gaps(nrows);
    const float* cen[3] = {cx.data(), cy.data(), cz.data()};
    // Entries left under kMaxGridEntries for the whole image; a tree whose
    // lists would pass it keeps no grid (its points take the tree BVH).
    const uint64_t have = img_->ur_cell_prims.size();
    const uint64_t budget = have < kMaxGridEntries ? kMaxGridEntries - have : 0;
    std::atomic<uint64_t> produced{0};
    std::atomic<bool> over{false};
    auto work = [&](int item) {
      const int by = item % nby, bz = item / nby;
      std::vector<int32_t> near, cands;
      std::vector<std::pair<double, int32_t>> cand;
      near.reserve(np);
      cands.reserve(np);
      cand.reserve(64);
      for (int bx = 0; bx < nbx; ++bx) {
        if (over.load(std::memory_order_relaxed)) return;
        uint64_t block_entries = 0;
        const int i0[3] = {bx * blk, by * blk, bz * blk};
        const int i1[3] = {std::min(i0[0] + blk, dims[0]), std::min(i0[1] + blk, dims[1]),
                           std::min(i0[2] + blk, dims[2])};
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) extent(a, i0[a], i1[a], &lo[a], &hi[a]);
        double bound = std::numeric_limits<double>::infinity();
        for (int k = 0; k < np; ++k) {
          double f2 = 0.0;
          for (int a = 0; a < 3; ++a) {
            double f = std::max(std::fabs(double(cen[a][k]) - lo[a]), std::fabs(double(cen[a][k]) - hi[a]));
            f2 += f * f;
          }
          double f = std::sqrt(f2);
          bound = std::min(bound, rho[k] >= 0.0f ? f - rho[k] : f + 2.0 * rad[k]);
        }
        bound += slack + 1e-9 * std::fabs(bound);
        double thr_max = std::max(double(t.r), bound) * (1.0 + 1e-5) + 1e-6;
        thr_max += slack + 1e-9 * thr_max;
        const double thr_max2 = thr_max * thr_max;
        near.clear();
        cands.clear();
        for (int k = 0; k < np; ++k) {
          double l2 = 0.0, g2 = 0.0;
          for (int a = 0; a < 3; ++a) {
            double c = double(cen[a][k]);
            double d = std::max({0.0, lo[a] - c, c - hi[a]}) + half;
            l2 += d * d;
            double gap = std::max({0.0, double(pb[k].mn[a]) - hi[a], lo[a] - double(pb[k].mx[a])});
            g2 += gap * gap;
          }
          double l = std::sqrt(l2);
          if ((rho[k] >= 0.0f ? l - rho[k] : l + 2.0 * rad[k]) < bound) near.push_back(k);
          if (g2 < thr_max2) cands.push_back(k);
        }
        for (int z = i0[2]; z < i1[2]; ++z)
          for (int y = i0[1]; y < i1[1]; ++y) {
            const size_t row = static_cast<size_t>(z) * dims[1] + y;
            auto& offs = row_offsets[row];
            auto& prims = row_prims[row];
            auto& gaps = row_gaps[row];
            for (int x = i0[0]; x < i1[0]; ++x) {
              double mn[3], mx[3];
              const int idx[3] = {x, y, z};
              for (int a = 0; a < 3; ++a) extent(a, idx[a], idx[a] + 1, &mn[a], &mx[a]);
              double min_ub = std::numeric_limits<double>::infinity();
              for (int32_t k : near) {
                double fx = std::max(std::fabs(double(cx[k]) - mn[0]), std::fabs(double(cx[k]) - mx[0]));
                double fy = std::max(std::fabs(double(cy[k]) - mn[1]), std::fabs(double(cy[k]) - mx[1]));
                double fz = std::max(std::fabs(double(cz[k]) - mn[2]), std::fabs(double(cz[k]) - mx[2]));
                double far = std::sqrt(fx * fx + fy * fy + fz * fz);
                double u = rho[k] >= 0.0f ? far - rho[k] : far + 2.0 * rad[k];
                min_ub = std::min(min_ub, u);
              }
              // slack of 1e-5 keeps float rounding of the device-side bound on the safe side
              double thr = std::max(double(t.r), min_ub) * (1.0 + 1e-5) + 1e-6;
              double thr2 = thr * thr;
              cand.clear();
              for (int32_t k : cands) {
                double g2 = 0.0;
                for (int a = 0; a < 3; ++a) {
                  double gap = std::max({0.0, double(pb[k].mn[a]) - mx[a], mn[a] - double(pb[k].mx[a])});
                  g2 += gap * gap;
                }
                if (g2 < thr2) cand.emplace_back(g2, k);
              }
              // Sorted by box gap, so the device meets the likely nearest
              // primitive first and prunes the rest.
              std::sort(cand.begin(), cand.end());
              offs.push_back(static_cast<uint32_t>(prims.size()));
              block_entries += cand.size();
              for (const auto& c : cand) {
                prims.push_back(c.second);
                // Points of the cell are at least pad inside the padded box, so
                // the device's float box bound of any of them exceeds this value.
                gaps.push_back(std::nextafter(static_cast<float>(std::sqrt(c.first) * (1.0 - 1e-6)), 0.0f));
              }
            }
          }
        if (produced.fetch_add(block_entries) + block_entries > budget) over.store(true);
      }
    };
    // Columns of blocks are independent: they are built on worker threads and
    // the rows concatenated in cell order.
    const int items = nby * nbz;
    unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    nthreads = std::min<unsigned>(nthreads, static_cast<unsigned>(items));
    std::atomic<int> next{0};
    // A worker's exception (a failed allocation) stops the others and is
    // rethrown here once all have ended; if no thread can be started, the
    // calling thread does the work.
    std::exception_ptr failure;
    std::mutex failure_mu;
    // Workers start together once all are running.  Each, and the calling
    // thread, which rethrows a worker's failure, first touches the C++
    // runtime's per-thread exception state: glibc allocates a loaded
    // library's thread-local block on first use and aborts the process when
    // that allocation fails, so it must not first happen in a throw after
    // the workers have used up the memory.
    (void)std::uncaught_exceptions();
    std::atomic<bool> go{false};
    auto drain = [&]() {
      (void)std::uncaught_exceptions();
      while (!go.load(std::memory_order_acquire)) std::this_thread::yield();
      try {
        for (int it = next.fetch_add(1); it < items; it = next.fetch_add(1)) work(it);
      } catch (...) {
        std::lock_guard<std::mutex> lock(failure_mu);
        if (!failure) failure = std::current_exception();
        over.store(true);
      }
    };
    std::vector<std::thread> pool;
    pool.reserve(nthreads);
    for (unsigned i = 0; i < nthreads; ++i) {
      try {
        pool.emplace_back(drain);
      } catch (...) {  // no thread (system_error) or no memory for its state
        break;
      }
    }
    go.store(true, std::memory_order_release);
    if (pool.empty()) drain();
    for (auto& th : pool) th.join();
    if (failure) std::rethrow_exception(failure);
    if (over.load()) return false;
    *cell_first = static_cast<int32_t>(img_->ur_cell_offsets.size());
    for (size_t row = 0; row < nrows; ++row) {
      uint32_t base = static_cast<uint32_t>(img_->ur_cell_prims.size());
      for (uint32_t o : row_offsets[row]) img_->ur_cell_offsets.push_back(base + o);
      img_->ur_cell_prims.insert(img_->ur_cell_prims.end(), row_prims[row].begin(), row_prims[row].end());
      img_->ur_cell_gaps.insert(img_->ur_cell_gaps.end(), row_gaps[row].begin(), row_gaps[row].end());
      for (int32_t pos : row_prims[row]) img_->ur_cell_nodes.push_back(img_->ur_prims[t.prim_first + pos]);
    }
    img_->ur_cell_offsets.push_back(static_cast<uint32_t>(img_->ur_cell_prims.size()));
    return true;
  }

  bool build_urtree(HostLeaf& leaf, float r, int depth) {
    HostUrTree t;
    std::memset(&t, 0, sizeof(t));
    t.r = r;
    t.depth = depth;
    t.prim_first = static_cast<int32_t>(img_->ur_prims.size());
    // In-order positions and inner nodes.
    std::function<int(int)> walk = [&](int i) -> int {
      const ft_node& n = d_.nodes[i];
      if (is_prim(n.kind)) {
        int posn = static_cast<int>(img_->ur_prims.size()) - t.prim_first;
        img_->ur_prims.push_back(i);
        return -(posn + 1);
      }
      int self = static_cast<int>(img_->ur_inner.size());
      img_->ur_inner.push_back(HostUrInner{{0, 0}, 0, 0});
      int lo = static_cast<int>(img_->ur_prims.size()) - t.prim_first;
      int a = walk(n.a);
      int b = walk(n.b);
      int hi = static_cast<int>(img_->ur_prims.size()) - t.prim_first;
      img_->ur_inner[self] = HostUrInner{{a, b}, lo, hi};
      return self;
    };
    t.inner_root = walk(leaf.node);
    t.n_prims = static_cast<int32_t>(img_->ur_prims.size()) - t.prim_first;
    // Parent links (the device folds one or two near primitives up to the
    // root along them).
    img_->ur_inner_up.resize(img_->ur_inner.size(), -1);
    img_->ur_prim_up.resize(img_->ur_prims.size(), -1);
    if (t.inner_root >= 0) {
      for (size_t in = static_cast<size_t>(t.inner_root); in < img_->ur_inner.size(); ++in)
        for (int side = 0; side < 2; ++side) {
          int32_t c = img_->ur_inner[in].child[side];
          int32_t link = static_cast<int32_t>(in << 1) | side;
          if (c >= 0) img_->ur_inner_up[c] = link;
          else img_->ur_prim_up[t.prim_first + (-c - 1)] = link;
        }
    }
    // Static material-model mixing of each inner node's primitives.
    img_->ur_inner_blend.resize(img_->ur_inner.size(), 0);
    for (size_t in = static_cast<size_t>(t.inner_root); in < img_->ur_inner.size(); ++in) {
      const HostUrInner& u = img_->ur_inner[in];
      int model = -1;
      int32_t mixed = 0;
      for (int k = u.lo; k < u.hi; ++k) {
        int mk = material_kind(img_->nodes[img_->ur_prims[t.prim_first + k]].material_id);
        if (model < 0) model = mk;
        else if (mk != model) mixed = 1;
      }
      img_->ur_inner_blend[in] = mixed;
    }
    std::vector<int32_t> pos(t.n_prims);
    std::iota(pos.begin(), pos.end(), 0);
    t.bvh_root = build_ur_bvh(pos, 0, pos.size(), t.prim_first);
    build_ur_grid(t);
    if (!emit_program(leaf.node, &t.fallback_first, &t.fallback_count)) return false;
    leaf.kind = kLeafUrTree;
    leaf.first = static_cast<int32_t>(img_->urtrees.size());
    leaf.count = t.n_prims;
    img_->urtrees.push_back(t);
    return true;
  }

  bool classify(size_t li) {
    HostLeaf& leaf = img_->leaves[li];
    const ft_node& n = d_.nodes[leaf.node];
    if (is_prim(n.kind)) {
      leaf.kind = kLeafPrim;
      leaf.first = leaf.count = 0;
      return true;
    }
    float r;
    int np, depth;
    if (is_urtree(leaf.node, &r, &np, &depth)) return build_urtree(leaf, r, depth);
    leaf.kind = kLeafGeneric;
    return emit_program(leaf.node, &leaf.first, &leaf.count);
  }
};

}  // namespace

bool build_scene_image(const ft_scene_desc& desc, SceneImage* out, std::string* error) {
  *out = SceneImage{};
  Builder b(desc, out, error);
  return b.run();
}

// parse_camera (R:6263-6286) + PinholeCamera::generate_ray basis
// (crates/forgedthoughts/src/render_api.rs:132-144), all in f32.
CameraBasis camera_basis(const float org[3], const float tgt[3], float fov) {
  auto normalize = [](float v[3]) {
    float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l <= std::numeric_limits<float>::epsilon()) return;
    float s = 1.0f / l;
    v[0] *= s;
    v[1] *= s;
    v[2] *= s;
  };
  auto cross = [](const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  CameraBasis cb;
  std::memcpy(cb.origin, org, sizeof(cb.origin));
  float up0[3] = {0.0f, 1.0f, 0.0f};
  float f[3] = {tgt[0] - org[0], tgt[1] - org[1], tgt[2] - org[2]};
  normalize(f);
  float r[3];
  cross(f, up0, r);
  normalize(r);
  float u[3];
  cross(r, f, u);
  normalize(u);
  std::memcpy(cb.forward, f, sizeof(f));
  std::memcpy(cb.right, r, sizeof(r));
  std::memcpy(cb.up, u, sizeof(u));
  cb.tan_fov = std::tan(0.5f * deg_to_rad(fov));
  return cb;
}

CameraBasis resolve_camera(const SceneImage& img, const ft_render_options& opt) {
  float org[3] = {img.scene_center[0], img.scene_center[1], img.scene_center[2] + opt.camera_z};
  float tgt[3] = {img.scene_center[0], img.scene_center[1], img.scene_center[2]};
  float fov = opt.fov_y_degrees;
  if (img.has_camera) {
    if (!std::isnan(img.camera.origin[0])) std::memcpy(org, img.camera.origin, sizeof(org));
    if (!std::isnan(img.camera.target[0])) std::memcpy(tgt, img.camera.target, sizeof(tgt));
    if (!std::isnan(img.camera.fov_y_degrees)) fov = img.camera.fov_y_degrees;
  }
  return camera_basis(org, tgt, fov);
}

}  // namespace ftgpu

// ------------------------------------------------------------ parameters
namespace {

bool param_prim(const ft_node& n) { return n.kind == FT_NODE_SPHERE || n.kind == FT_NODE_BOX; }

// union_round trees reachable from the root, each as (root node, in-order
// primitives); false with `error` when a tree holds something the adjoint
// does not differentiate.
bool param_trees(const ft_scene_desc& d, std::vector<std::pair<int, std::vector<int>>>* trees, std::string* error) {
  std::vector<std::pair<int, int>> stack{{d.root, -1}};  // (node, parent kind)
  std::vector<char> seen(d.n_nodes, 0);
  while (!stack.empty()) {
    auto [i, parent_kind] = stack.back();
    stack.pop_back();
    if (i < 0 || static_cast<uint32_t>(i) >= d.n_nodes || seen[i]) continue;
    seen[i] = 1;
    const ft_node& n = d.nodes[i];
    if (n.kind == FT_NODE_UNION_ROUND && parent_kind != FT_NODE_UNION_ROUND) {
      std::vector<int> prims;
      std::vector<int> walk{i};
      // in-order: left subtree first
      std::function<bool(int)> rec = [&](int k) -> bool {
        if (k < 0 || static_cast<uint32_t>(k) >= d.n_nodes) return false;
        const ft_node& m = d.nodes[k];
        if (m.kind == FT_NODE_UNION_ROUND) return rec(m.a) && rec(m.b);
        if (!param_prim(m)) {
          *error = "union_round tree holds a node kind the adjoint does not differentiate";
          return false;
        }
        bool shell = m.kind == FT_NODE_SPHERE ? m.f[1] != 0.0f : (m.f[3] != 0.0f || m.f[4] != 0.0f);
        if (shell || m.rot_deg[0] != 0.0f || m.rot_deg[2] != 0.0f) {
          *error = "differentiable primitives need no x / z rotation, rounding or shell";
          return false;
        }
        prims.push_back(k);
        return true;
      };
      if (!rec(i)) {
        if (error->empty()) *error = "malformed union_round tree";
        return false;
      }
      trees->emplace_back(i, std::move(prims));
      continue;
    }
    if (n.kind >= FT_NODE_UNION && n.kind != FT_NODE_SLICE && n.kind != FT_NODE_SMOOTH) {
      stack.push_back({n.b, n.kind});
      stack.push_back({n.a, n.kind});
    }
  }
  return true;
}

float* param_field(ft_node& n, int field) {
  switch (field) {
    case FT_PARAM_CX: return &n.center[0];
    case FT_PARAM_CY: return &n.center[1];
    case FT_PARAM_CZ: return &n.center[2];
    case FT_PARAM_ROT_Y: return &n.rot_deg[1];
    case FT_PARAM_S0: return &n.f[0];
    case FT_PARAM_S1: return &n.f[1];
    case FT_PARAM_S2: return &n.f[2];
    case FT_PARAM_RADIUS: return &n.f[0];
    default: return nullptr;
  }
}

bool check_param(const ft_scene_desc& d, const ft_param& p) {
  if (p.node < 0 || static_cast<uint32_t>(p.node) >= d.n_nodes || p.field < 0 || p.field > FT_PARAM_RADIUS) return false;
  const ft_node& n = d.nodes[p.node];
  return p.field == FT_PARAM_RADIUS ? n.kind == FT_NODE_UNION_ROUND : param_prim(n);
}

}  // namespace

extern "C" {

ft_status ft_scene_param_layout(const ft_scene_desc* desc, uint32_t capacity, ft_param* params, uint32_t* count) {
  FT_API_BEGIN
  if (!desc || !count || (capacity && !params))
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "desc, count and params must be non-null");
  if (desc->root < 0 || static_cast<uint32_t>(desc->root) >= desc->n_nodes || !desc->nodes)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "invalid scene description");
  std::vector<std::pair<int, std::vector<int>>> trees;
  std::string err;
  if (!param_trees(*desc, &trees, &err)) return ftcommon::fail(FT_ERR_UNSUPPORTED, err);
  std::vector<ft_param> out;
  for (const auto& tr : trees) {
    for (int prim : tr.second)
      for (int f = FT_PARAM_CX; f <= FT_PARAM_S2; ++f) out.push_back(ft_param{prim, f});
    out.push_back(ft_param{tr.first, FT_PARAM_RADIUS});
  }
  *count = static_cast<uint32_t>(out.size());
  for (uint32_t i = 0; i < std::min<uint32_t>(capacity, *count); ++i) params[i] = out[i];
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_desc_get_params(const ft_scene_desc* desc, const ft_param* params, uint32_t n, float* values) {
  FT_API_BEGIN
  if (!desc || (n && (!params || !values))) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "null argument");
  for (uint32_t i = 0; i < n; ++i) {
    if (!check_param(*desc, params[i]))
      return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "parameter " + std::to_string(i) + " is not differentiable");
    values[i] = *param_field(const_cast<ft_node&>(desc->nodes[params[i].node]), params[i].field);
  }
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_desc_set_params(ft_scene_desc* desc, const ft_param* params, uint32_t n, const float* values) {
  FT_API_BEGIN
  if (!desc || (n && (!params || !values))) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "null argument");
  for (uint32_t i = 0; i < n; ++i)
    if (!check_param(*desc, params[i]) || !std::isfinite(values[i]))
      return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "parameter " + std::to_string(i) + " is invalid");
  for (uint32_t i = 0; i < n; ++i) {
    if (params[i].field == FT_PARAM_RADIUS) {
      std::vector<int> stack{params[i].node};
      while (!stack.empty()) {
        int k = stack.back();
        stack.pop_back();
        if (k < 0 || static_cast<uint32_t>(k) >= desc->n_nodes) continue;
        // descriptions are library- or caller-owned writable arrays behind a const view
        ft_node& m = const_cast<ft_node&>(desc->nodes[k]);
        if (m.kind != FT_NODE_UNION_ROUND) continue;
        m.f[0] = values[i];
        stack.push_back(m.a);
        stack.push_back(m.b);
      }
    } else {
      *param_field(const_cast<ft_node&>(desc->nodes[params[i].node]), params[i].field) = values[i];
    }
  }
  return FT_OK;
  FT_API_END
}

}  // extern "C"
