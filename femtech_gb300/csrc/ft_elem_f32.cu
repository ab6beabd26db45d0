// ft_elem_f32.cu -- float instantiations of the element kernels and their launcher.
#include "ft_elem.cuh"
#include "ft_launch.h"

namespace ftgpu {

template <int ET, int MAT>
static int go(int gp, int nb, int th, size_t sm, cudaStream_t s, const ElemArgs<float> &A, int dto) {
  // C3D8 blocks of more than 128 elements need more than 48 KB of shared
  // memory (the geometry records); allowed once per device, at the first
  // launch there (set-up)
  static bool opted[64] = {};
  int dev = 0;
  if (ET == 0 && (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64))
    return (int)cudaErrorInvalidDevice;
  if (ET == 0 && !opted[dev]) {
    const int mx = (int)elem_smem_bytes_host<float>(0, kMaxPatchElems);
    for (cudaError_t e : {cudaFuncSetAttribute(k_elem<float, ET, MAT, true, false>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, mx),
                          cudaFuncSetAttribute(k_elem<float, ET, MAT, false, true>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, mx),
                          cudaFuncSetAttribute(k_elem<float, ET, MAT, false, false>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, mx)})
      if (e != cudaSuccess) return (int)e;
    opted[dev] = true;
  }
  if (gp == kLaunchGaussPoints)
    k_elem<float, ET, MAT, true, false><<<nb, th, sm, s>>>(A, dto);
  else if (gp == kLaunchInjury)
    k_elem<float, ET, MAT, false, true><<<nb, th, sm, s>>>(A, dto);
  else
    k_elem<float, ET, MAT, false, false><<<nb, th, sm, s>>>(A, dto);
  return (int)cudaGetLastError();
}

template <int ET>
static int by_mat(int mat, int gp, int nb, int th, size_t sm, cudaStream_t s,
                  const ElemArgs<float> &A, int dto) {
  switch (mat) {
    case 0: return go<ET, 0>(gp, nb, th, sm, s, A, dto);
    case 1: return go<ET, 1>(gp, nb, th, sm, s, A, dto);
    case 2: return go<ET, 2>(gp, nb, th, sm, s, A, dto);
    case 3: return go<ET, 3>(gp, nb, th, sm, s, A, dto);
    case 4: return go<ET, 4>(gp, nb, th, sm, s, A, dto);
    case 5: return go<ET, 5>(gp, nb, th, sm, s, A, dto);
    case 6: return go<ET, 6>(gp, nb, th, sm, s, A, dto);
    case 7: return go<ET, 7>(gp, nb, th, sm, s, A, dto);
    default: return (int)cudaErrorInvalidValue;
  }
}

int launch_strain_f32(int etype, int nblocks, int threads, size_t smem, cudaStream_t s,
                      const ElemArgs<float> &A, double *Eout) {
  if (nblocks <= 0) return 0;
  if (etype == 0)
    k_elem_strain<float, 0><<<nblocks, threads, smem, s>>>(A, Eout);
  else
    k_elem_strain<float, 1><<<nblocks, threads, smem, s>>>(A, Eout);
  return (int)cudaGetLastError();
}

int launch_geo_f32(int nblocks, cudaStream_t s, const ElemArgs<float> &A, float *geo) {
  if (nblocks <= 0) return 0;
  k_elem_geo<float><<<nblocks, 128, 0, s>>>(A, geo);
  return (int)cudaGetLastError();
}

int launch_elem_f32(int etype, int mat, int gp, int nblocks, int threads, size_t smem,
                    cudaStream_t s, const ElemArgs<float> &A, int dt_only) {
  if (nblocks <= 0) return 0;
  return etype == 0 ? by_mat<0>(mat, gp, nblocks, threads, smem, s, A, dt_only)
                    : by_mat<1>(mat, gp, nblocks, threads, smem, s, A, dt_only);
}

}  // namespace ftgpu
