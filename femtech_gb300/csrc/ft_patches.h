// ft_patches.h -- host-side mesh partitioning into element patches.
#pragma once

#include <cstdint>
#include <vector>

namespace ftgpu {

struct PatchGroup {
  int etype;        // 0 C3D8, 1 C3D4
  int mat;          // material ID
  int patch_begin;  // first patch
  int npatch;
  int elem_begin;   // first element (group order)
  int nelem;
};

// Result of build_patches.  "Group order" is the element order used on the
// device: elements sorted by (type, material, instance, Morton code).
struct PatchSet {
  std::vector<PatchGroup> groups;
  std::vector<int> elem_order;      // group order -> reference element index
  std::vector<int> patch_elem_off;  // [P+1]
  std::vector<int> patch_node_off;  // [P+1] slot offsets
  std::vector<int> patch_inst;      // [P]
  std::vector<int> patch_ent_off;   // [P+1]
  std::vector<uint16_t> lptr;       // per patch: n_local+1 offsets
  std::vector<uint16_t> lent;       // local CSR entries (e_local * NC + corner)
  std::vector<uint16_t> lconn;      // per group: nelem*NC local corner nodes
  std::vector<long long> group_lconn_off;  // per group: start in lconn (multiple of 8)
  std::vector<int> slot_node;       // [S] global node of each slot
  std::vector<int> node_slot_off;   // [N+1]
  std::vector<int> node_slots;      // node -> slots, ascending
};

// Build patches of at most `max_elems` elements and `max_nodes` local nodes.
// elem_inst: instance of each element; elem_mat: material of each element.
// Returns 0 or a negative status (element not in one instance, bad input).
int build_patches(int nNodes, int nelements, const double *coordinates, const int *eptr,
                  const int *connectivity, const int *etype, const int *elem_mat,
                  const int *elem_inst, int max_elems, int max_nodes, PatchSet &out);

}  // namespace ftgpu
