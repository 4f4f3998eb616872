// Host-side lattice set-up: reference BC masks and the device flag words.
#pragma once
#include <stdint.h>

#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "lbm_types.h"

namespace lbm {

// The reference's BC masks of the nodes its BC file lists (2D masks use the
// low 32 bits), in ascending node order: per boundary node b, the mask, the
// pulls its streaming flags block (bit d) and the link directions its BC file
// lists (bit dir).  Every other node has a zero mask and blocks nothing.
struct RefMasks {
    int q = 9;
    std::vector<long long> bc_nodes;  // nodes with at least one link, ascending
    std::vector<uint64_t> mask;
    std::vector<uint32_t> blocked;
    std::vector<uint32_t> linked;
};

// Allocator whose resize leaves new elements uninitialised, for per-node
// host arrays that the builders fill in parallel anyway.
template <class T>
struct NoInitAllocator : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAllocator<U>;
    };
    NoInitAllocator() = default;
    template <class U>
    NoInitAllocator(const NoInitAllocator<U> &) {}
    template <class U>
    void construct(U *p) {
        ::new ((void *)p) U;
    }
    template <class U, class... A>
    void construct(U *p, A &&...a) {
        ::new ((void *)p) U(std::forward<A>(a)...);
    }
};
template <class T>
using HostArray = std::vector<T, NoInitAllocator<T>>;

// What the step kernel reads: one flag word per node, and for special nodes
// a slot with the reference mask (reference mode) or the face kind (physics).
struct DeviceFlags {
    HostArray<uint32_t> word;
    HostArray<int32_t> slot;
    std::vector<uint64_t> mask;
    std::vector<int32_t> kind;
    std::vector<long long> slot_node;
};

int lattice_cx(int q, int d);
int lattice_cy(int q, int d);
int lattice_cz(int q, int d);
int lattice_opp(int q, int d);
// Link type of direction dir, main type and corner bit of boundary node b.
uint64_t ref_type(const RefMasks &r, size_t b, int dir);
uint64_t ref_main_type(const RefMasks &r, size_t b);
bool ref_corner(const RefMasks &r, size_t b);
// Place of a node in the boundary-node list, or -1.
long long find_bc(const RefMasks &r, long long node);

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
