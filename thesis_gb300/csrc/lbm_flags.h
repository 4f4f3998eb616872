// Host-side lattice set-up: reference BC masks and the device flag words.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "lbm_types.h"

namespace lbm {

// The reference's per-node BC masks (2D masks use the low 32 bits) and, per
// node, the pulls its streaming flags block (bit d) and the link directions
// its BC file lists (bit dir).
struct RefMasks {
    int q = 9;
    std::vector<uint64_t> mask;
    std::vector<uint32_t> blocked;
    std::vector<uint32_t> linked;
    std::vector<long long> bc_nodes;  // nodes with at least one link, ascending
};

// What the step kernel reads: one flag word per node, and for special nodes
// a slot with the reference mask (reference mode) or the face kind (physics).
struct DeviceFlags {
    std::vector<uint32_t> word;
    std::vector<int32_t> slot;
    std::vector<uint64_t> mask;
    std::vector<int32_t> kind;
    std::vector<long long> slot_node;
};

int lattice_cx(int q, int d);
int lattice_cy(int q, int d);
int lattice_cz(int q, int d);
int lattice_opp(int q, int d);
uint64_t ref_type(const RefMasks &r, int node, int dir);
uint64_t ref_main_type(const RefMasks &r, int node);
bool ref_corner(const RefMasks &r, int node);

int build_ref_masks(const lbm_lattice_desc &L, RefMasks &r, std::string &err);
// Reference curved walls in effect: reference mode, CURVED boundary type and
// the simple wall model (the reference's HH wall kernel has no curved branch).
bool curved_walls(const lbm_params &P, int q);
// Boundary conditions only the one-node kernels apply (the shared boundary
// code): curved walls and the reference's 2D extrapolation outlets.
bool one_node_boundaries(const lbm_params &P, int q);
int build_device_flags(const lbm_lattice_desc &L, const lbm_params &P, const RefMasks &r,
                       DeviceFlags &out, std::string &err);

}  // namespace lbm
