// Connected-component colours of the volume fraction on one periodic block:
// the resetcolor, union-find recolor and propagate stages of
// Vof::MakeIteration (src/solver/vof.ipp:546-578) with
// UVof::Imp::RecolorUnionFind (src/util/vof.ipp:982-1150), same results.
//
//   components  gas cells (u > 0.5), listed by one pass over the field and
//               then walked from the list alone, 26-connected across the
//               periodic boundaries, by a lock-free union-find: a root is only ever
//               hooked under a smaller root (atomicCAS), so each
//               component's root is its first cell in x-fastest order, the
//               cell whose unique initial colour the reference keeps;
//   stable map  per component, the previous colour of its first cell in
//               the order of the cells with two halo layers that has one
//               (atomicMin of that order's 64-bit index);
//   reduction   on the host over the components (few): the stable colour
//               unless already given, else the next unused one;
//   propagate   cells without colour with 0 < u take the colour of a face
//               neighbour with larger u, faces in the mesh's order.  Faces of
//               one direction that share no cell lie on different lines
//               along that direction, and within a line only the runs of
//               such cells (with the faces on both sides) can change, so
//               one thread replays one run in order; halo cells hold the
//               colours from before the pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <set>
#include <vector>

#include "common.cuh"

namespace aphgpu {
namespace {

constexpr int kLabelThreads = 256;
constexpr int kMaxComponents = 1 << 21;
constexpr unsigned long long kNoFirst = ~0ull;
constexpr long long kNoColorBits = 0xBFF0000000000000LL;  // -1.0, no colour

__device__ __forceinline__ int Wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Root of x (bounded walk; the tree depth is below the cell count), with
// path halving: each visited cell is pointed at its grandparent (as in the
// ECL-CC labelling of Jaiganesh and Burtscher).  A cell that is not a root
// has a smaller parent, and only roots are ever hooked, so the grandparent
// is an ancestor of the cell whatever the other threads do, and a plain
// store cannot lose a hooking.
__device__ __forceinline__ int Find(volatile int* par, int x, int64_t cap) {
  for (int64_t it = 0; it < cap; ++it) {
    const int p = par[x];
    if (p == x) return x;
    const int gp = par[p];
    if (gp != p) par[x] = gp;
    x = gp;
  }
  return x;
}

__device__ __forceinline__ bool Gas(double u) { return u > 0.5; }

// warp-aggregated append of c to the list when `want` (every lane of the
// warp calls it)
__device__ __forceinline__ void Append(bool want, int c, int* list, int* count) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (want) list[base + __popc(m & ((1u << lane) - 1u))] = c;
}

// the gas cells, listed, each with an initial parent: the gas cell before
// it along z, else along y, else along x (no wrap: a smaller index, in the
// same component), else itself, as ECL-CC initialises its parents with a
// smaller neighbour, so the unions start from trees already joined (par of the other cells is never read: gas is tested on u).  The
// loop bound is uniform over each warp.
__global__ void KLabelInit(int64_t n, int nx, int ny, const double* __restrict__ u, int* par,
                           int* list, int* count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c0 = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); c0 < n;
       c0 += stride) {
    const int64_t c = c0 + (threadIdx.x & 31);
    const bool g = c < n && Gas(u[c]);
    if (g) {
      const int64_t nxy = (int64_t)nx * ny;
      int p = (int)c;
      if (c % nx != 0 && Gas(u[c - 1])) p = (int)(c - 1);
      if ((c / nx) % ny != 0 && Gas(u[c - nx])) p = (int)(c - nx);
      if (c >= nxy && Gas(u[c - nxy])) p = (int)(c - nxy);
      par[c] = p;
    }
    Append(g, (int)c, list, count);
  }
}

// Union of every listed gas cell with its gas neighbours in the 13 offsets
// of one half of the 3x3x3 stencil (the other half is the same pairs
// reversed).
__global__ void KLabelUnion(Dims d, const double* __restrict__ u, int* par,
                            const int* __restrict__ gas, const int* gcount, int* err) {
  const int64_t n = d.cells();
  const int ng = *gcount;
  volatile int* vp = par;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
    const int64_t c = gas[t];
    const int i = (int)(c % d.nx), j = (int)((c / d.nx) % d.ny), k = (int)(c / ((int64_t)d.nx * d.ny));
    for (int o = 0; o < 13; ++o) {
      // offsets with dz > 0, or dz == 0 and dy > 0, or dz == dy == 0, dx > 0
      const int q = o + 14;  // 14..26 in the 27-point numbering
      const int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = q / 9 - 1;
      const int64_t cn = d.idx(Wrap(i + dx, d.nx), Wrap(j + dy, d.ny), Wrap(k + dz, d.nz));
      if (cn == c || !Gas(u[cn])) continue;
      int a = (int)c, b = (int)cn;
      bool done = false;
      for (int it = 0; it < (1 << 20) && !done; ++it) {
        a = Find(vp, a, n);
        b = Find(vp, b, n);
        if (a == b) {
          done = true;
        } else {
          if (a < b) {
            const int t2 = a;
            a = b;
            b = t2;
          }
          // hook the larger root under the smaller, if still a root
          if (atomicCAS(&par[a], a, b) == a) done = true;
        }
      }
      if (!done) atomicExch(err, 1);
    }
  }
}

// Roots of the listed gas cells; each root gets a component slot.
__global__ void KLabelFlatten(int64_t n, int* par, const int* __restrict__ gas,
                              const int* gcount, int* slot, int* ncomp, int* croot, int cap,
                              int* err) {
  volatile int* vp = par;
  const int ng = *gcount;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
    const int c = gas[t];
    const int r = Find(vp, c, n);
    if (r == c) {
      const int s = atomicAdd(ncomp, 1);
      if (s < cap) {
        slot[c] = s;
        croot[s] = c;
      } else {
        atomicExch(err, 2);
      }
    }
  }
}

__global__ void KLabelRoot(int64_t n, int* par, const int* __restrict__ gas, const int* gcount) {
  volatile int* vp = par;
  const int ng = *gcount;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
    const int c = gas[t];
    par[c] = Find(vp, c, n);
  }
}

// The first position, in the order of the cells with two halo layers
// (x-fastest over [-2, n+2) per axis), of a gas cell of each component that
// has a previous colour.  A cell's smallest position takes its left halo
// copy where it has one (the last two cells of an axis).
__global__ void KLabelFirst(Dims d, const int* __restrict__ root, const int* __restrict__ slot,
                            const int* __restrict__ gas, const int* gcount,
                            const double* __restrict__ clprev, unsigned long long* first) {
  const unsigned long long ex = d.nx + 4, ey = d.ny + 4;
  const int ng = *gcount;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  // the loop bound is uniform over each warp; the listed cells of a warp
  // are consecutive gas cells, mostly of one component: their minimum is
  // formed in the warp and written by one atomic
  for (int t0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); t0 < ng; t0 += stride) {
    const int t = t0 + lane;
    unsigned long long e = kNoFirst;
    int s = -1;
    if (t < ng) {
      const int64_t c = gas[t];
      if (clprev[c] != -1.0) {
        const int i = (int)(c % d.nx), j = (int)((c / d.nx) % d.ny),
                  k = (int)(c / ((int64_t)d.nx * d.ny));
        const int xi = i >= d.nx - 2 ? i - d.nx + 2 : i + 2;
        const int yj = j >= d.ny - 2 ? j - d.ny + 2 : j + 2;
        const int zk = k >= d.nz - 2 ? k - d.nz + 2 : k + 2;
        e = ((unsigned long long)zk * ey + yj) * ex + xi;
        s = slot[root[c]];
      }
    }
    const unsigned want = __ballot_sync(0xffffffffu, s >= 0);
    if (!want) continue;
    // lanes without a candidate take the first candidate's slot and a
    // neutral position, so that one component in the warp matches all
    const int s0 = __shfl_sync(0xffffffffu, s, __ffs(want) - 1);
    const int sv = s >= 0 ? s : s0;
    int all = 0;
    __match_all_sync(0xffffffffu, sv, &all);
    // the stored minimum only decreases: an atomic that could not lower it
    // is skipped (a read through L2 first), so most of a component's cells
    // issue none
    if (all) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, e, o);
        e = v < e ? v : e;
      }
      if (lane == 0 && e < __ldcg(&first[s0])) atomicMin(&first[s0], e);
    } else if (s >= 0 && e < __ldcg(&first[s])) {
      atomicMin(&first[s], e);
    }
  }
}

// Previous colour at each component's first position.
__global__ void KLabelStable(Dims d, int nc, const unsigned long long* __restrict__ first,
                             const double* __restrict__ clprev, double* stable) {
  const unsigned long long ex = d.nx + 4, ey = d.ny + 4;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nc; s += gridDim.x * blockDim.x) {
    const unsigned long long e = first[s];
    if (e == kNoFirst) {
      stable[s] = -1.0;
      continue;
    }
    const int i = Wrap((int)(e % ex) - 2, d.nx);
    const int j = Wrap((int)((e / ex) % ey) - 2, d.ny);
    const int k = Wrap((int)(e / (ex * ey)) - 2, d.nz);
    stable[s] = clprev[d.idx(i, j, k)];
  }
}

// New colours, and their copy from before the propagation pass on the
// cells at the ends of the lines (the only ones it reads there).  The cells
// the propagation may colour (no colour, u > 0: the candidates) are marked
// in `cand` and listed.  A CTA walks rows (y, z) of the grid (row = y + ny
// z), two cells of a row per thread with 16-byte loads and stores (nx
// even; else one cell per thread).
__device__ __forceinline__ double ApplyCell(int64_t c, double uc, const int* __restrict__ root,
                                            const int* __restrict__ slot,
                                            const double* __restrict__ color) {
  return Gas(uc) ? color[slot[root[c]]] : -1.0;
}
// Append over the active lanes of a warp
__device__ __forceinline__ void AppendActive(bool want, int c, int* list, int* count) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, want);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(m));
  base = __shfl_sync(act, base, leader);
  if (want) list[base + __popc(m & ((1u << lane) - 1u))] = c;
}
__global__ void KLabelApply(Dims d, const int* __restrict__ root, const int* __restrict__ slot,
                            const double* __restrict__ color, const double* __restrict__ u,
                            double* cl, double* pre, unsigned char* cand, int* clist,
                            int* ccount) {
  const int per = (d.nx % 2 == 0) ? 2 : 1;
  const int nrows = d.ny * d.nz;
  for (int row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int y = row % d.ny, z = row / d.ny;
    const int64_t base = (int64_t)row * d.nx;
    const bool edge_yz = y == 0 || y == d.ny - 1 || z == 0 || z == d.nz - 1;
    for (int x0 = per * (blockIdx.y * blockDim.x + threadIdx.x); x0 < d.nx;
         x0 += per * gridDim.y * blockDim.x) {
      const int64_t c = base + x0;
      double u2[2], v2[2];
      if (per == 2) {
        const double2 uu = *reinterpret_cast<const double2*>(u + c);
        u2[0] = uu.x;
        u2[1] = uu.y;
        v2[0] = ApplyCell(c, u2[0], root, slot, color);
        v2[1] = ApplyCell(c + 1, u2[1], root, slot, color);
        *reinterpret_cast<double2*>(cl + c) = make_double2(v2[0], v2[1]);
      } else {
        u2[0] = u[c];
        v2[0] = ApplyCell(c, u2[0], root, slot, color);
        cl[c] = v2[0];
      }
      for (int e = 0; e < per; ++e) {
        const int x = x0 + e;
        if (edge_yz || x == 0 || x == d.nx - 1) pre[c + e] = v2[e];
        const bool cd = v2[e] == -1.0 && u2[e] > 0;
        cand[c + e] = cd ? 1 : 0;
        AppendActive(cd, (int)(c + e), clist, ccount);
      }
    }
  }
}

// The faces of direction `dir` of one line, in order: face w lies between
// the line's cells w-1 and w; at w = 0 and w = m the outer cell is the
// halo copy of the line's other end, with the colour from before the pass.
// A face changes a colour only where one of its cells is a candidate (no
// colour, u > 0), and a cell that is not one never changes (its colour is
// set, or u <= 0), so the faces of a line split into independent runs: each
// maximal run of consecutive candidates with the faces on both sides of it.
// A thread replays the run that starts at a listed candidate whose previous
// cell along `dir` is not one (or at the line's first cell, whose previous
// cell is the halo copy), in face order, exactly as the whole line's replay
// would.
__global__ void KLabelPropagate(Dims d, int dir, const double* __restrict__ u, double* cl,
                                const double* __restrict__ pre,
                                const unsigned char* __restrict__ cand,
                                const int* __restrict__ clist, const int* ccount) {
  const int m = dir == 0 ? d.nx : dir == 1 ? d.ny : d.nz;
  const int64_t stride = dir == 0 ? 1 : dir == 1 ? (int64_t)d.nx : (int64_t)d.nx * d.ny;
  const int n = *ccount;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int64_t c = clist[t];
    const int64_t x = c % d.nx, y = (c / d.nx) % d.ny, z = c / ((int64_t)d.nx * d.ny);
    const int w0 = (int)(dir == 0 ? x : dir == 1 ? y : z);
    const int64_t base = c - (int64_t)w0 * stride;  // the line's first cell
    if (w0 > 0 && cand[c - stride]) continue;  // not the start of its run
    const int64_t last = base + (int64_t)(m - 1) * stride;
    double cl0, u0;
    if (w0 == 0) {
      cl0 = pre[last];  // halo copy before cell 0
      u0 = u[last];
    } else {
      cl0 = cl[c - stride];
      u0 = u[c - stride];
    }
    // faces w0 .. (the run's last cell) + 1
    for (int w = w0; w <= m; ++w) {
      const int64_t c1 = base + (int64_t)w * stride;
      double cl1;
      double u1;
      bool in_run;
      if (w < m) {
        cl1 = cl[c1];
        u1 = u[c1];
        in_run = cand[c1] != 0;
      } else {
        cl1 = pre[base];  // halo copy after the last cell
        u1 = u[base];
        in_run = false;
      }
      // the comparisons on the bit patterns (integer instructions): in each
      // rule one operand of u0 > u1 / u1 > u0 is positive, and for a
      // positive double and any other non-NaN double the signed 64-bit
      // order of the bits is the numeric order; -1 (no colour) has one bit
      // pattern
      const long long b0 = __double_as_longlong(u0), b1 = __double_as_longlong(u1);
      bool none0 = __double_as_longlong(cl0) == kNoColorBits;
      const bool none1 = __double_as_longlong(cl1) == kNoColorBits;
      if (none0 && b0 > 0 && b1 > b0 && !none1) {
        cl0 = cl1;
        none0 = false;
        if (w > 0) cl[c1 - stride] = cl0;
      }
      if (none1 && b1 > 0 && b0 > b1 && !none0) {
        cl1 = cl0;
        if (w < m) cl[c1] = cl1;
      }
      cl0 = cl1;
      u0 = u1;
      if (!in_run) break;  // the face after the run's last cell is done
    }
  }
}

__global__ void KColorInit(int64_t n, const double* __restrict__ u, double* cl) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    cl[c] = u[c] > 0 ? 0.0 : -1.0;
}

int Blocks(int64_t n) { return FlatBlocks(n); }

}  // namespace

// Colours as the reference's Vof starts them from a zero colour field:
// 0 where u > 0, none elsewhere (src/solver/vof.ipp:53-57).
int ColorInit(aphgpu_ctx* ctx) {
  const int64_t N = ctx->N;
  if (!ctx->cl) APH_TRY(Alloc(ctx, &ctx->cl, N));
  KColorInit<<<Blocks(N), kLabelThreads, 0, ctx->stream>>>(N, ctx->u, ctx->cl);
  APH_LAUNCHED(ctx);
  return APHGPU_OK;
}

int Recolor(aphgpu_ctx* ctx) {
  const Dims d = ctx->d;
  const int64_t N = ctx->N;
  cudaStream_t st = ctx->stream;
  auto& L = ctx->lab;
  if (!L.par) {
    APH_TRY(Alloc(ctx, &L.par, N));
    APH_TRY(Alloc(ctx, &L.gas, N));
    APH_TRY(Alloc(ctx, &L.slot, N));
    APH_TRY(Alloc(ctx, &L.croot, kMaxComponents));
    APH_TRY(Alloc(ctx, &L.first, kMaxComponents));
    APH_TRY(Alloc(ctx, &L.stable, kMaxComponents));
    APH_TRY(Alloc(ctx, &L.color, kMaxComponents));
    APH_TRY(Alloc(ctx, &L.pre, N));
    APH_TRY(Alloc(ctx, &L.ctl, 4));
    APH_TRY(Alloc(ctx, &L.flag, N));
  }
  const int nb = Blocks(N);
  APH_CUDA(ctx, cudaMemsetAsync(L.ctl, 0, 4 * sizeof(int), st));
  int* gcount = L.ctl + 2;
  KLabelInit<<<nb, kLabelThreads, 0, st>>>(N, d.nx, d.ny, ctx->u, L.par, L.gas, gcount);
  APH_LAUNCHED(ctx);
  // the list passes: a grid of 8 CTAs per SM looping over the gas cells
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
      sms < 1) {
    cudaGetLastError();
    sms = 152;
  }
  const int lb = 8 * sms;
  KLabelUnion<<<lb, kLabelThreads, 0, st>>>(d, ctx->u, L.par, L.gas, gcount, L.ctl + 1);
  APH_LAUNCHED(ctx);
  KLabelFlatten<<<lb, kLabelThreads, 0, st>>>(N, L.par, L.gas, gcount, L.slot, L.ctl, L.croot,
                                              kMaxComponents, L.ctl + 1);
  APH_LAUNCHED(ctx);
  KLabelRoot<<<lb, kLabelThreads, 0, st>>>(N, L.par, L.gas, gcount);
  APH_LAUNCHED(ctx);
  int hc[2] = {0, 0};
  APH_CUDA(ctx, cudaMemcpyAsync(hc, L.ctl, sizeof(hc), cudaMemcpyDeviceToHost, st));
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  if (hc[1] == 1) return SetError(ctx, APHGPU_ERR_TIMEOUT, "recolor: union did not settle");
  if (hc[1] == 2 || hc[0] > kMaxComponents)
    return SetError(ctx, APHGPU_ERR_UNSUPPORTED, "recolor: more than %d components",
                    kMaxComponents);
  const int nc = hc[0];
  std::vector<double> color(std::max(nc, 1));
  if (nc > 0) {
    APH_CUDA(ctx, cudaMemsetAsync(L.first, 0xff, sizeof(unsigned long long) * nc, st));
    KLabelFirst<<<lb, kLabelThreads, 0, st>>>(d, L.par, L.slot, L.gas, gcount, ctx->cl, L.first);
    APH_LAUNCHED(ctx);
    KLabelStable<<<Blocks(nc), kLabelThreads, 0, st>>>(d, nc, L.first, ctx->cl, L.stable);
    APH_LAUNCHED(ctx);
    std::vector<int> croot(nc);
    std::vector<double> stable(nc);
    APH_CUDA(ctx, cudaMemcpyAsync(croot.data(), L.croot, sizeof(int) * nc, cudaMemcpyDeviceToHost, st));
    APH_CUDA(ctx, cudaMemcpyAsync(stable.data(), L.stable, sizeof(double) * nc,
                                  cudaMemcpyDeviceToHost, st));
    APH_CUDA(ctx, cudaStreamSynchronize(st));
    // ReduceColor over the components in the order of their first cells
    std::vector<int> order(nc);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return croot[a] < croot[b]; });
    double next = 0;
    for (int s = 0; s < nc; ++s)
      if (stable[s] != -1.0) next = std::max(next, stable[s]);
    next += 1;
    std::set<double> used;
    for (int s : order) {
      if (stable[s] == -1.0 || used.count(stable[s])) {
        color[s] = next;
        next += 1;
      } else {
        color[s] = stable[s];
      }
      used.insert(color[s]);
    }
    APH_CUDA(ctx, cudaMemcpyAsync(L.color, color.data(), sizeof(double) * nc,
                                  cudaMemcpyHostToDevice, st));
  }
  // the candidates of the propagation, listed in the gas list's storage
  // (the union-find passes are done with it) and counted in ctl[3]
  int* ccount = L.ctl + 3;
  {
    // CTAs of 256 threads, each over rows of up to 512 cells (more CTAs
    // per row along y for longer rows), 16 per SM
    const int rows = d.ny * d.nz;
    const dim3 g((unsigned)std::min(rows, 16 * sms), (unsigned)((d.nx + 511) / 512));
    KLabelApply<<<g, 256, 0, st>>>(d, L.par, L.slot, L.color, ctx->u, ctx->cl, L.pre, L.flag,
                                   L.gas, ccount);
  }
  APH_LAUNCHED(ctx);
  for (int dir = 0; dir < 3; ++dir) {
    KLabelPropagate<<<lb, kLabelThreads, 0, st>>>(d, dir, ctx->u, ctx->cl, L.pre, L.flag, L.gas,
                                                  ccount);
    APH_LAUNCHED(ctx);
  }
  // the host vector of colours stays alive until the copy has completed
  APH_CUDA(ctx, cudaStreamSynchronize(st));
  return APHGPU_OK;
}

}  // namespace aphgpu
