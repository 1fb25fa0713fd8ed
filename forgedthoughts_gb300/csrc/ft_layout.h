// Device-image layout constants shared by the host scene builder and the
// kernels (including kernels compiled at run time): leaf kinds, generic-leaf
// opcodes and the fixed capacities of the evaluators.  No host headers.
#pragma once

#include "forgedthoughts_gb300.h"

namespace ftgpu {

// Leaf kinds.
enum LeafKind : int32_t {
  kLeafPrim = 0,     // a single primitive node: inline evaluation
  kLeafGeneric = 1,  // postfix program over the leaf's node tree
  kLeafUrTree = 2    // union_round tree of primitives with one radius
};

// Generic-program opcodes (top 5 bits of a uint32 op word, node index below).
enum GenericOp : uint32_t {
  kGPrim = 0,        // push primitive distance at the current point
  kGDomainPush = 1,  // q = domain(to_local(p)); push point
  kGLocalPush = 2,   // q = to_local(p); push point (distance_post / noise)
  kGPostPop = 3,     // d = distance_post(d, p); pop point
  kGNoisePop = 4,    // d = noise(p, d); pop point
  kGPop = 5,         // pop point (after a domain base)
  kGBinary = 6,      // combine the two top values with the node's operator
  kGSlice = 7,
  kGSmooth = 8,
  kGCustom = 9       // push a user `sdf` definition's distance at the current point
};
constexpr uint32_t kGOpShift = 27;
constexpr uint32_t kGNodeMask = (1u << kGOpShift) - 1u;
constexpr int kMaxGenericValueStack = 16;
constexpr int kMaxGenericPointStack = 8;
constexpr int kMaxUrDepth = 40;
constexpr int kUrNear = 8;       // near-set capacity of the union_round tree path
constexpr int kUrBvhLeafSize = 4;
// Iteration cap of the device's stack walks over trees (BVHs, union_round
// inner nodes): a valid tree pops each node once, so this only ends a walk
// over a corrupted one.
constexpr int kMaxWalk = 1 << 20;

}  // namespace ftgpu
