// ft_noalloc.cu -- a C3D8 internal-force entry point that allocates nothing.
//
// Who needs it: drivers that own every byte of device memory themselves and
// cannot let a library call cudaMalloc/cudaFree -- for instance a coupled
// solver that hands all device memory to its own pool allocator, a caller
// running under a fixed memory budget, or a loop that must not hit the
// implicit device synchronisation of cudaFree.  They pass device arrays in
// the reference's layout and get the assembled internal force back in a
// device array they own.
//
// How: the per-element corner forces (the scratch between the element pass
// and the deterministic node gather) live in one file-scope __device__ array
// of FTGPU_NOALLOC_MAX_ELEMENTS * 24 doubles.  Every GPU that loads this
// library holds that array until the process exits.  Host code cannot use
// the array's name as a device address, so the first call on each device
// looks the address up with cudaGetSymbolAddress (with that device current)
// and passes it to the kernels.  The address is cached per device index for
// the life of that device's primary context: after cudaDeviceReset it is
// stale.  Every call reads the error word back and waits for its stream, so
// the call cannot be captured into a CUDA graph.  All calls share the one
// array: two calls that overlap on the GPU (different streams, or different
// host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "ft_elem.cuh"
#include "ftgpu.h"

namespace ftgpu {

static __device__ __align__(256) double g_noalloc_corner_force[FTGPU_NOALLOC_MAX_ELEMENTS * 24];

// The error word of the call also lives in static device memory: bit 0 = an
// inverted or non-finite element, bit 1 = a node -> corner entry outside
// [0, 8 * nelements).
static __device__ int g_noalloc_bad;

constexpr int kNoAllocMaxDevices = 64;
static double *g_noalloc_ptr[kNoAllocMaxDevices];
static int *g_noalloc_bad_ptr[kNoAllocMaxDevices];
static std::mutex g_noalloc_mu;

// One thread per element: the C3D8 element force of ft_elem.cuh in FP64,
// reading coordinates/displacements straight from the caller's AoS arrays.
template <int MAT>
__global__ void k_noalloc_hex(int nelements, const double *X, const int *conn, const double *u,
                              MatP<double> mp, double *corner, int *bad_out) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelements) return;
  double x[8][3], uu[8][3];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int n = conn[8 * e + a];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      x[a][d] = X[3 * n + d];
      uu[a][d] = u[3 * n + d];
    }
  }
  ElemArgs<double> none;
  memset(&none, 0, sizeof(none));
  const double pc[4] = {0, 0, 0, 0};
  const double a0[3] = {1, 0, 0};
  double f[8][3], le;
  int bad = 0;
  hex_element<double, MAT, false, false>(x, uu, mp, pc, a0, nullptr, 0, 0, false, f, le, bad,
                                         none, 0, nullptr, 0);
  if (bad) atomicOr(bad_out, 1);
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d) corner[24ll * e + 3 * a + d] = f[a][d];
}

// One thread per node: fi = sum of its corners, in the caller's CSR order.
// An entry outside this call's corners is skipped and flagged (bit 1), so a
// bad map can neither read another call's leftovers nor run off the array.
__global__ void k_noalloc_gather(int nNodes, int nelements, const int *ptr, const int *ent,
                                 const double *corner, double *fi, int *bad_out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nNodes) return;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  const int k1 = ptr[n + 1];
  for (int k = ptr[n]; k < k1; ++k) {
    const int c8 = ent[k];
    if (c8 < 0 || c8 >= 8 * nelements) {
      atomicOr(bad_out, 2);
      continue;
    }
    const long long c = 3ll * c8;
    s0 += corner[c];
    s1 += corner[c + 1];
    s2 += corner[c + 2];
  }
  fi[3 * n] = s0;
  fi[3 * n + 1] = s1;
  fi[3 * n + 2] = s2;
}

}  // namespace ftgpu

using namespace ftgpu;

extern "C" int ftgpu_hex8_force_noalloc(int nNodes, int nelements, const double *coordinates,
                                        const int *connectivity, const int *node_elem_ptr,
                                        const int *node_elem_ent, const double *u, int materialID,
                                        const double *properties, double *fi, void *stream) {
  if (nelements <= 0 || nNodes <= 0 || !coordinates || !connectivity || !node_elem_ptr ||
      !node_elem_ent || !u || !properties || !fi)
    return FTGPU_ERR_INPUT;
  if (nelements > FTGPU_NOALLOC_MAX_ELEMENTS) return FTGPU_ERR_INPUT;
  if (materialID == 5 || materialID == 7) return FTGPU_ERR_INPUT;  // history needs state
  if (materialID < 0 || materialID > 7) return FTGPU_ERR_MATERIAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
    return FTGPU_ERR_NODEVICE;
  double *scratch = nullptr;
  int *bad = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      // set-up, once per device, with that device current
      void *p = nullptr, *pb = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_corner_force) != cudaSuccess || !p ||
          cudaGetSymbolAddress(&pb, g_noalloc_bad) != cudaSuccess || !pb) {
        cudaGetLastError();
        return FTGPU_ERR_CUDA;
      }
      g_noalloc_ptr[dev] = static_cast<double *>(p);
      g_noalloc_bad_ptr[dev] = static_cast<int *>(pb);
    }
    scratch = g_noalloc_ptr[dev];
    bad = g_noalloc_bad_ptr[dev];
  }
  // Parameters as the model's set-up builds them for FP64 mode; Ogden in
  // FP64 always takes the eigen-decomposition (ser_thr2 = 0, no series).
  MatP<double> mp;
  memset(&mp, 0, sizeof(mp));
  for (int k = 0; k < 9; ++k) mp.p[k] = properties[k];
  mp.K = properties[2] + 2.0 * properties[1] / 3.0;
  mp.mat = materialID;
  mp.ser_thr2 = 0.0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemsetAsync(bad, 0, sizeof(int), s) != cudaSuccess) return FTGPU_ERR_CUDA;
  const int th = 128, nb = (nelements + th - 1) / th;
  // One case per law of StressUpdate.cpp:7-27 (plus Ogden); the two
  // viscoelastic laws were rejected above.
  switch (materialID) {
    case 0: k_noalloc_hex<0><<<nb, th, 0, s>>>(nelements, coordinates, connectivity, u, mp, scratch, bad); break;
    case 1: k_noalloc_hex<1><<<nb, th, 0, s>>>(nelements, coordinates, connectivity, u, mp, scratch, bad); break;
    case 2: k_noalloc_hex<2><<<nb, th, 0, s>>>(nelements, coordinates, connectivity, u, mp, scratch, bad); break;
    case 3: k_noalloc_hex<3><<<nb, th, 0, s>>>(nelements, coordinates, connectivity, u, mp, scratch, bad); break;
    case 4: k_noalloc_hex<4><<<nb, th, 0, s>>>(nelements, coordinates, connectivity, u, mp, scratch, bad); break;
    case 6: k_noalloc_hex<6><<<nb, th, 0, s>>>(nelements, coordinates, connectivity, u, mp, scratch, bad); break;
    default: return FTGPU_ERR_MATERIAL;
  }
  if (cudaGetLastError() != cudaSuccess) return FTGPU_ERR_CUDA;
  k_noalloc_gather<<<(nNodes + 255) / 256, 256, 0, s>>>(nNodes, nelements, node_elem_ptr,
                                                        node_elem_ent, scratch, fi, bad);
  if (cudaGetLastError() != cudaSuccess) return FTGPU_ERR_CUDA;
  int hbad = 0;
  if (cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return FTGPU_ERR_CUDA;
  if (hbad & 2) return FTGPU_ERR_INPUT;
  return hbad ? FTGPU_ERR_INVERTED : FTGPU_OK;
}
