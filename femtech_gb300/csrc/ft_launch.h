// ft_launch.h -- host launchers of the element kernels (one translation unit per precision).
#pragma once

#include <cuda_runtime.h>

#include "ft_common.h"
#include "ft_injury.cuh"

namespace ftgpu {

// Launch modes of the element kernel (argument gp of launch_elem_*)
enum { kLaunchPlain = 0, kLaunchGaussPoints = 1, kLaunchInjury = 2 };

// Launch the element kernel of (etype, material) over `nblocks` patches.
// gp = kLaunchGaussPoints records per-Gauss-point F/detF/PK2, kLaunchInjury
// also updates the injury criteria of the listed elements (force pass);
// dt_only = 1 computes only the stable-time-step contribution.  Returns a
// cudaError_t value.
int launch_elem_f32(int etype, int mat, int gp, int nblocks, int threads, size_t smem,
                    cudaStream_t s, const ElemArgs<float> &A, int dt_only);
int launch_elem_f64(int etype, int mat, int gp, int nblocks, int threads, size_t smem,
                    cudaStream_t s, const ElemArgs<double> &A, int dt_only);

// Element strain pass (k_elem_strain) of one group: Voigt Green strain per
// element into Eout (group order).  Returns a cudaError_t value.
int launch_strain_f32(int etype, int nblocks, int threads, size_t smem, cudaStream_t s,
                      const ElemArgs<float> &A, double *Eout);
int launch_strain_f64(int etype, int nblocks, int threads, size_t smem, cudaStream_t s,
                      const ElemArgs<double> &A, double *Eout);
template <class R>
inline int launch_strain(int etype, int nblocks, int threads, size_t smem, cudaStream_t s,
                         const ElemArgs<R> &A, double *Eout);
template <>
inline int launch_strain<float>(int etype, int nblocks, int threads, size_t smem, cudaStream_t s,
                                const ElemArgs<float> &A, double *Eout) {
  return launch_strain_f32(etype, nblocks, threads, smem, s, A, Eout);
}
template <>
inline int launch_strain<double>(int etype, int nblocks, int threads, size_t smem,
                                 cudaStream_t s, const ElemArgs<double> &A, double *Eout) {
  return launch_strain_f64(etype, nblocks, threads, smem, s, A, Eout);
}

// Setup pass of an FP32 C3D8 group (k_elem_geo): the Gauss points' inverse
// reference Jacobians and determinants into geo ([20][nelem] x 4 values).
// Returns a cudaError_t value.
int launch_geo_f32(int nblocks, cudaStream_t s, const ElemArgs<float> &A, float *geo);

// Dynamic shared memory of one element block: node X and u records (4
// values each) for kMaxLocalNodes slots plus NC*3 corner forces per element, or for FP32
// C3D8 the larger 80-value geometry record per element in the same space.
template <class R>
inline size_t elem_smem_bytes_host(int etype, int PE) {
  const int NC = etype == 0 ? 8 : 4;
  const size_t per_elem = (etype == 0 && sizeof(R) == 4) ? 80 : (size_t)NC * 3;
  const size_t slot_words = etype == 0 ? 8 : 6;  // packed records (C3D8) / component arrays
  return sizeof(R) * (slot_words * (size_t)kMaxLocalNodes + per_elem * PE) +
         (etype == 0 ? elem_csr_smem_bytes(NC, PE) : 0);
}

// Dynamic shared memory of one strain block (k_elem_strain): the slot
// records only.
template <class R>
inline size_t strain_smem_bytes_host() {
  return sizeof(R) * 8 * (size_t)kMaxLocalNodes;
}

template <class R>
inline int launch_elem(int etype, int mat, int gp, int nblocks, int threads, size_t smem,
                       cudaStream_t s, const ElemArgs<R> &A, int dt_only);
template <>
inline int launch_elem<float>(int etype, int mat, int gp, int nblocks, int threads, size_t smem,
                              cudaStream_t s, const ElemArgs<float> &A, int dt_only) {
  return launch_elem_f32(etype, mat, gp, nblocks, threads, smem, s, A, dt_only);
}
template <>
inline int launch_elem<double>(int etype, int mat, int gp, int nblocks, int threads,
                               size_t smem, cudaStream_t s, const ElemArgs<double> &A,
                               int dt_only) {
  return launch_elem_f64(etype, mat, gp, nblocks, threads, smem, s, A, dt_only);
}

}  // namespace ftgpu
