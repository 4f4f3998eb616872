// Internal constants shared by host and device code.
#pragma once
#include <stdint.h>

#include "thesis_lbm.h"

namespace lbm {

// Per-node flag word, one uint32 per lattice node:
//   bit 0        fluid node (the reference's fluid_d == 1)
//   bits 1..18   pull of population d is blocked (the reference's stream flag
//                for direction d cleared, or, in physics mode, x - c_d is
//                solid or outside a non-periodic domain)
//   bit 19       special node: boundary handling needs its slot record
constexpr uint32_t W_FLUID = 1u;
constexpr uint32_t W_SPECIAL = 1u << 19;

// Physics-mode slot kinds (bc_kind): face id in bits 0..2 (inward normal
// 0 +x, 1 -x, 2 +y, 3 -y, 4 +z, 5 -z), pressure face, outlet face, active.
constexpr int BCK_FACE_MASK = 7;
constexpr int BCK_PRESSURE = 8;
constexpr int BCK_OUTLET = 16;
constexpr int BCK_ACTIVE = 32;
// A velocity face whose prescribed velocity is tangential to it is a moving
// wall: half-way bounce-back with the momentum of the wall added on the
// links listed (bit d: incoming direction d) in the slot's mask.
constexpr int BCK_MOVING = 64;
// Physics-mode open outlets on any face (the reference's OUTLET_FIRST,
// OUTLET_SECOND and OUTLET_HEmodel, GpuBoundaries.cu:1562-1874, with the
// populations addressed per node): the populations entering through the face
// copied from the node one step inward (first order), extrapolated from the
// nodes one and two steps inward (second order), or set to the equilibrium
// of the node's own macroscopic state of the previous step (HEmodel).
constexpr int BCK_EXTRAP1 = 128;
constexpr int BCK_EXTRAP2 = 256;
constexpr int BCK_HE = 512;

}  // namespace lbm
