// Stencil helpers shared by the single-domain and the batched solvers:
// operator access on the compact storage (couplings to the minus
// neighbours, optional explicit diagonal) and the tile loop of the stencil
// kernels.
#pragma once

#include "common.cuh"

namespace aphgpu {


template <class T>
struct Op {
  Dims d;
  const T* w0;
  const T* w1;
  const T* w2;
  const T* diag;  // may be NULL: -(sum of the six couplings)
};

// Couplings of cell (i,j,k) in reference order xm,xp,ym,yp,zm,zp.
template <class T>
__device__ __forceinline__ void Couplings(const Op<T>& A, int i, int j, int k,
                                          int64_t c, T e[6]) {
  const Dims& d = A.d;
  const int ip = wrapp(i + 1, d.nx), jp = wrapp(j + 1, d.ny), kp = wrapp(k + 1, d.nz);
  e[0] = A.w0[c];
  e[1] = A.w0[d.idx(ip, j, k)];
  e[2] = A.w1[c];
  e[3] = A.w1[d.idx(i, jp, k)];
  e[4] = A.w2[c];
  e[5] = A.w2[d.idx(i, j, kp)];
}

template <class T>
__device__ __forceinline__ T Diag(const Op<T>& A, int64_t c, const T e[6]) {
  if (A.diag) return A.diag[c];
  T s = T(0);
  s += e[0];
  s += e[1];
  s += e[2];
  s += e[3];
  s += e[4];
  s += e[5];
  return -s;
}

// sum_q e_q x_nb(q) + e0 x_c, in the order of linear.ipp:66-72
template <class T>
__device__ __forceinline__ T Apply(const Op<T>& A, const T* x, int i, int j,
                                   int k, int64_t c) {
  const Dims& d = A.d;
  T e[6];
  Couplings(A, i, j, k, c, e);
  const T e0 = Diag(A, c, e);
  const int im = wrapm(i - 1, d.nx), ip = wrapp(i + 1, d.nx);
  const int jm = wrapm(j - 1, d.ny), jp = wrapp(j + 1, d.ny);
  const int km = wrapm(k - 1, d.nz), kp = wrapp(k + 1, d.nz);
  T u = x[c] * e0;
  u += x[d.idx(im, j, k)] * e[0];
  u += x[d.idx(ip, j, k)] * e[1];
  u += x[d.idx(i, jm, k)] * e[2];
  u += x[d.idx(i, jp, k)] * e[3];
  u += x[d.idx(i, j, km)] * e[4];
  u += x[d.idx(i, j, kp)] * e[5];
  return u;
}

#define TILE_LOOP_BEGIN(dims)                                    \
  const int i = blockIdx.x * kTileX + threadIdx.x;               \
  const int j = blockIdx.y * kTileY + threadIdx.y;               \
  const int kb = blockIdx.z * kTileZ;                            \
  const int ke = min(kb + kTileZ, (dims).nz);                    \
  const bool inxy = i < (dims).nx && j < (dims).ny;              \
  for (int k = kb; k < ke; ++k) {                                \
    if (!inxy) continue;                                         \
    const int64_t c = (dims).idx(i, j, k);
#define TILE_LOOP_END }

template <class T>
Op<T> MakeOp(const Level<T>& L) {
  return Op<T>{L.d, L.w[0], L.w[1], L.w[2], L.has_diag ? L.diag : nullptr};
}

}  // namespace aphgpu
