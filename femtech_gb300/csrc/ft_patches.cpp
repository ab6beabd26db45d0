// ft_patches.cpp -- partition the mesh into element patches (host, once per model).
//
// The reference keeps one flat element loop (GetForce_3D.cpp:15) and adds each
// element's force into the global array.  Here elements are sorted by
// (element type, material, instance, Morton code of the centroid) and cut
// greedily into patches that fit one thread block: at most max_elems elements
// and max_nodes distinct nodes.  Each patch owns a contiguous range of "slots"
// (one per local node) holding replicated reference coordinates and
// displacements and receiving the patch's partial nodal forces.  Two CSR maps
// make the sums deterministic: per patch, local node -> (element, corner) in
// element order; per node, node -> slots in ascending slot order.
#include "ft_patches.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace ftgpu {

static inline uint64_t spread21(uint64_t v) {
  v &= 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

int build_patches(int nNodes, int nelements, const double *X, const int *eptr, const int *conn,
                  const int *etype, const int *elem_mat, const int *elem_inst, int max_elems,
                  int max_nodes, PatchSet &out) {
  out = PatchSet();
  if (nelements <= 0 || nNodes <= 0) return -3;
  // bounding box for the Morton codes
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int n = 0; n < nNodes; ++n)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], X[3 * n + d]);
      hi[d] = std::max(hi[d], X[3 * n + d]);
    }
  double ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
  if (!(ext > 0)) ext = 1.0;
  const double scale = 2097151.0 / ext;
  struct Key {
    uint64_t hi, lo;
    int e;
  };
  std::vector<Key> keys(nelements);
  for (int e = 0; e < nelements; ++e) {
    const int nn = eptr[e + 1] - eptr[e];
    if ((etype[e] == 0 && nn != 8) || (etype[e] == 1 && nn != 4) || etype[e] < 0 || etype[e] > 1)
      return -3;
    double c[3] = {0, 0, 0};
    for (int k = eptr[e]; k < eptr[e + 1]; ++k) {
      const int n = conn[k];
      if (n < 0 || n >= nNodes) return -3;
      for (int d = 0; d < 3; ++d) c[d] += X[3 * n + d];
    }
    uint64_t q[3];
    for (int d = 0; d < 3; ++d) {
      double v = (c[d] / nn - lo[d]) * scale;
      q[d] = (uint64_t)std::min(2097151.0, std::max(0.0, v));
    }
    uint64_t morton = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
    // hi: type (1 bit) | material (8 bits) | instance (24 bits)
    uint64_t h = ((uint64_t)etype[e] << 40) | ((uint64_t)(elem_mat[e] & 0xff) << 32) |
                 (uint64_t)(uint32_t)elem_inst[e];
    keys[e] = Key{h, morton, e};
  }
  std::stable_sort(keys.begin(), keys.end(), [](const Key &a, const Key &b) {
    return a.hi != b.hi ? a.hi < b.hi : a.lo < b.lo;
  });

  std::vector<int> stamp(nNodes, -1), lidx(nNodes, 0);
  out.elem_order.resize(nelements);
  out.patch_elem_off.push_back(0);
  out.patch_node_off.push_back(0);
  out.patch_ent_off.push_back(0);
  std::vector<int> local_nodes;     // of the current patch
  std::vector<int> cur_elems;
  int p = 0;
  long long slot_base = 0;
  int egroup = 0;
  auto flush = [&](int NC) {
    // local CSR: local node -> (element, corner) entries, in element order
    const int nl = (int)local_nodes.size();
    std::vector<int> cnt(nl + 1, 0);
    for (int le = 0; le < (int)cur_elems.size(); ++le) {
      const int e = cur_elems[le];
      for (int a = 0; a < NC; ++a) cnt[lidx[conn[eptr[e] + a]] + 1]++;
    }
    for (int i = 0; i < nl; ++i) cnt[i + 1] += cnt[i];
    std::vector<uint16_t> ent(cnt[nl]);
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int le = 0; le < (int)cur_elems.size(); ++le) {
      const int e = cur_elems[le];
      for (int a = 0; a < NC; ++a) ent[pos[lidx[conn[eptr[e] + a]]]++] = (uint16_t)(le * NC + a);
    }
    for (int i = 0; i <= nl; ++i) out.lptr.push_back((uint16_t)cnt[i]);
    out.lent.insert(out.lent.end(), ent.begin(), ent.end());
    for (int i = 0; i < nl; ++i) out.slot_node.push_back(local_nodes[i]);
    slot_base += nl;
    out.patch_node_off.push_back((int)slot_base);
    out.patch_elem_off.push_back(egroup);
    out.patch_ent_off.push_back((int)out.lent.size());
    out.patch_inst.push_back(elem_inst[cur_elems[0]]);
    local_nodes.clear();
    cur_elems.clear();
    ++p;
  };

  size_t k = 0;
  while (k < keys.size()) {
    // one group: same type and material
    const int e_first = keys[k].e;
    PatchGroup g;
    g.etype = etype[e_first];
    g.mat = elem_mat[e_first];
    g.patch_begin = p;
    g.elem_begin = egroup;
    const int NC = g.etype == 0 ? 8 : 4;
    // align the group's lconn block to 16 bytes
    while (out.lconn.size() % 8) out.lconn.push_back(0);
    out.group_lconn_off.push_back((long long)out.lconn.size());
    const uint64_t ghi = keys[k].hi >> 32;
    int cur_inst = -1;
    while (k < keys.size() && (keys[k].hi >> 32) == ghi) {
      const int e = keys[k].e;
      const int inst = elem_inst[e];
      int fresh = 0;
      for (int a = 0; a < NC; ++a) {
        const int n = conn[eptr[e] + a];
        if (stamp[n] != p) {
          bool dup = false;
          for (int b = 0; b < a; ++b)
            if (conn[eptr[e] + b] == n) dup = true;
          if (!dup) ++fresh;
        }
      }
      if (!cur_elems.empty() &&
          ((int)cur_elems.size() >= max_elems ||
           (int)local_nodes.size() + fresh > max_nodes || inst != cur_inst))
        flush(NC);
      cur_inst = inst;
      for (int a = 0; a < NC; ++a) {
        const int n = conn[eptr[e] + a];
        if (stamp[n] != p) {
          stamp[n] = p;
          lidx[n] = (int)local_nodes.size();
          local_nodes.push_back(n);
        }
        out.lconn.push_back((uint16_t)lidx[n]);
      }
      cur_elems.push_back(e);
      out.elem_order[egroup++] = e;
      ++k;
    }
    if (!cur_elems.empty()) flush(NC);
    g.npatch = p - g.patch_begin;
    g.nelem = egroup - g.elem_begin;
    out.groups.push_back(g);
  }
  // node -> slots (ascending slot order)
  out.node_slot_off.assign(nNodes + 1, 0);
  for (size_t s = 0; s < out.slot_node.size(); ++s) out.node_slot_off[out.slot_node[s] + 1]++;
  for (int n = 0; n < nNodes; ++n) out.node_slot_off[n + 1] += out.node_slot_off[n];
  out.node_slots.resize(out.slot_node.size());
  std::vector<int> pos(out.node_slot_off.begin(), out.node_slot_off.end() - 1);
  for (size_t s = 0; s < out.slot_node.size(); ++s) out.node_slots[pos[out.slot_node[s]]++] = (int)s;
  return 0;
}

}  // namespace ftgpu
