// ft_elem_f64.cu -- double instantiations of the element kernels and their launcher.
#include "ft_elem.cuh"
#include "ft_launch.h"

namespace ftgpu {

template <int ET, int MAT>
static int go(int gp, int nb, int th, size_t sm, cudaStream_t s, const ElemArgs<double> &A, int dto) {
  if (gp == kLaunchGaussPoints)
    k_elem<double, ET, MAT, true, false><<<nb, th, sm, s>>>(A, dto);
  else if (gp == kLaunchInjury)
    k_elem<double, ET, MAT, false, true><<<nb, th, sm, s>>>(A, dto);
  else
    k_elem<double, ET, MAT, false, false><<<nb, th, sm, s>>>(A, dto);
  return (int)cudaGetLastError();
}

template <int ET>
static int by_mat(int mat, int gp, int nb, int th, size_t sm, cudaStream_t s,
                  const ElemArgs<double> &A, int dto) {
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

int launch_strain_f64(int etype, int nblocks, int threads, size_t smem, cudaStream_t s,
                      const ElemArgs<double> &A, double *Eout) {
  if (nblocks <= 0) return 0;
  if (etype == 0)
    k_elem_strain<double, 0><<<nblocks, threads, smem, s>>>(A, Eout);
  else
    k_elem_strain<double, 1><<<nblocks, threads, smem, s>>>(A, Eout);
  return (int)cudaGetLastError();
}

int launch_elem_f64(int etype, int mat, int gp, int nblocks, int threads, size_t smem,
                    cudaStream_t s, const ElemArgs<double> &A, int dt_only) {
  if (nblocks <= 0) return 0;
  return etype == 0 ? by_mat<0>(mat, gp, nblocks, threads, smem, s, A, dt_only)
                    : by_mat<1>(mat, gp, nblocks, threads, smem, s, A, dt_only);
}

}  // namespace ftgpu
