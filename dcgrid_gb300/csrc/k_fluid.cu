// k_fluid.cu — field stages of the adaptive step: semi-Lagrangian advection
// (+ buoyancy / sources), divergence, Jacobi, prolongation, pressure gradient,
// fine-to-coarse restriction.
//
// Thread mapping: 256-thread CTAs, 4 blocks per CTA, one thread per cell; a
// warp covers half a block (4 subblocks, 32 contiguous floats = 128 B), so
// every field plane is read and written in full 128-byte lines.
#include "dcg_dev.cuh"
#include <algorithm>

#include "dcg_kernels.h"

namespace dcg {

// k_dcgrid_advect_velocity (dcgrid_fluid.cu:112-127) + buoyancy extension:
// v.y += dt * (-alpha * rho + beta * (T - T_amb)) on leaf cells.
__device__ __forceinline__ void advect_velocity_cell(const Dev &D, long long b, int c) {
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const size_t cell = (size_t)b * BV + c;
  float o0 = 0.f, o1 = 0.f, o2 = 0.f;
  if (D.child[cell >> 3] == NONE) {
    float px, py, pz;
    back_trace(D, bp, c, cell, px, py, pz);
    Smp s;
    sample_at(D, (uint32_t)b, bp, px, py, pz, s);
    if (!(s.wAcc < 1e-6f)) {
      const bool inside = box_inside(D.g, s);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        int x, y, z;
        corner_of(s, k, x, y, z);
        float vx = D.v[0][s.idx[k]], vy = D.v[1][s.idx[k]], vz = D.v[2][s.idx[k]];
        if (!inside) vel_bc(D.g, D.ph, vx, vy, vz, x, y, z, s.scale);
        if (k == 0) {
          o0 = vx * s.wt[0]; o1 = vy * s.wt[0]; o2 = vz * s.wt[0];
        } else {
          o0 = o0 + vx * s.wt[k]; o1 = o1 + vy * s.wt[k]; o2 = o2 + vz * s.wt[k];
        }
      }
    }
    if (D.ph.buoy_a != 0.f || D.ph.buoy_b != 0.f) {
      float f = -D.ph.buoy_a * q_ld(D, 0, cell);
      if (D.g.nq > 1) f = f + D.ph.buoy_b * (q_ld(D, 1, cell) - D.ph.t_amb);
      o1 = o1 + D.ph.dt * f;
    }
  }
  D.tv[0][cell] = o0;
  D.tv[1][cell] = o1;
  D.tv[2][cell] = o2;
}

// k_dcgrid_advect_density (dcgrid_fluid.cu:129-144) for every scalar; sphere
// sources (extension) overwrite leaf cells inside the source.
// Scalar storage with the format as a template argument (0 FP32, 1 BF16, 2 FP16).
template <int MODE> __device__ __forceinline__ float q_ldm(const Dev &D, int k, size_t i) {
  if (MODE == 0) return D.q[k][i];
  return h16_to_f(D.qh[k][i], MODE);
}
template <int MODE> __device__ __forceinline__ void tq_stm(const Dev &D, int k, size_t i, float v) {
  if (MODE == 0) D.tq[k][i] = v;
  else D.tqh[k][i] = f_to_h16(v, MODE);
}
// q_bc decided once per stencil corner for all scalars: 0 the sampled value
// passes, 1 inlet (density d_emit, other scalars 0), 2 zero
__device__ __forceinline__ int q_bc_mode(const Geom &g, const Phys &P, int x, int y, int z, int scale) {
  if (in_inlet(g, P, x, y, z, scale)) return 1;
  if (P.wind && yz_inside(g, y, z, scale)) {
    if (x < 0) return 2;
    if (x * scale >= g.gx) return 0;
  }
  return outside(g, x, y, z, scale) ? 2 : 0;
}

template <int MODE, int NQ>
__device__ __forceinline__ void advect_scalars_cell_t(const Dev &D, long long b, int c) {
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const size_t cell = (size_t)b * BV + c;
  float o[NQ];
#pragma unroll
  for (int kq = 0; kq < NQ; kq++) o[kq] = 0.f;
  if (D.child[cell >> 3] == NONE) {
    float px, py, pz;
    back_trace(D, bp, c, cell, px, py, pz);
    Smp s;
    sample_at(D, (uint32_t)b, bp, px, py, pz, s);
    if (!(s.wAcc < 1e-6f)) {
      // per scalar the sum runs over the corners in order, as in
      // k_dcgrid_advect_density (dcgrid_fluid.cu:129-144)
      const bool inside = box_inside(D.g, s);
#pragma unroll
      for (int k = 0; k < 8; k++) {
        int x, y, z;
        corner_of(s, k, x, y, z);
        const int mode = inside ? 0 : q_bc_mode(D.g, D.ph, x, y, z, s.scale);
#pragma unroll
        for (int kq = 0; kq < NQ; kq++) {
          const float qc = mode == 0 ? q_ldm<MODE>(D, kq, s.idx[k]) : (mode == 1 && kq == 0 ? D.ph.d_emit : 0.f);
          o[kq] = (k == 0) ? qc * s.wt[0] : o[kq] + qc * s.wt[k];
        }
      }
    }
    int lx, ly, lz;
    local_xyz(c, lx, ly, lz);
    if (D.ph.em_n > 0)
      o[0] = o[0] + D.ph.dt * emission_at(D.g, D.ph, bp.x + lx, bp.y + ly, bp.z + lz, 1 << bp.w);
    if (D.ph.src) {
      if (in_source(D.ph, bp.x + lx, bp.y + ly, bp.z + lz, 1 << bp.w))
#pragma unroll
        for (int kq = 0; kq < NQ; kq++) o[kq] = src_value_at(D.ph, kq, bp.x + lx, bp.y + ly, bp.z + lz, bp.w);
    }
  }
#pragma unroll
  for (int kq = 0; kq < NQ; kq++) tq_stm<MODE>(D, kq, cell, o[kq]);
}
__device__ __forceinline__ void advect_scalars_cell(const Dev &D, long long b, int c) {
  const int m = D.g.mixed;
  if (D.g.nq == 3) {
    if (m == 0) advect_scalars_cell_t<0, 3>(D, b, c);
    else if (m == 1) advect_scalars_cell_t<1, 3>(D, b, c);
    else advect_scalars_cell_t<2, 3>(D, b, c);
  } else {
    if (m == 0) advect_scalars_cell_t<0, 1>(D, b, c);
    else if (m == 1) advect_scalars_cell_t<1, 1>(D, b, c);
    else advect_scalars_cell_t<2, 1>(D, b, c);
  }
}

// Source cells set on every leaf cell (used once at initialisation).
__global__ void __launch_bounds__(256) k_sources(Dev D) {
  const long long b = (long long)blockIdx.x * 4 + (threadIdx.x >> 6);
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  if (in_source(D.ph, bp.x + lx, bp.y + ly, bp.z + lz, 1 << bp.w))
    for (int kq = 0; kq < D.g.nq; kq++) q_st(D, kq, cell, src_value_at(D.ph, kq, bp.x + lx, bp.y + ly, bp.z + lz, bp.w));
}

// Seeded velocity noise on every allocated cell.
__global__ void __launch_bounds__(256) k_add_noise(Dev D, unsigned long long seed, float amp) {
  const long long b = (long long)blockIdx.x * 4 + (threadIdx.x >> 6);
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  for (int d = 0; d < 3; d++)
    D.v[d][cell] = D.v[d][cell] + amp * noise_unit(seed, bp.x + lx, bp.y + ly, bp.z + lz, bp.w, d);
}

// accumulate<T> (dcgrid_structure.cu:188-205): parent cell = mean of the 8
// cells of the child subblock; one thread per subblock of one level.
__device__ __forceinline__ void restrict_subblock(const Dev &D, int level, const FieldList &fl, long long sl) {
  if (sl >= 8 * D.g.budget[level]) return;
  const long long b = D.g.off[level] + (sl >> 3);
  if (D.pos[b].w != level) return;
  const uint32_t par = D.parent[b];
  if (par == NONE) return;
  const int s = (int)(sl & 7);
  const size_t pc = (size_t)par * 8 + s;
  const size_t base = (size_t)b * BV + 8 * s;
  for (int f = 0; f < fl.n; f++) {
    float v[8];
    if (fl.mode[f] == 0) {
      const float *F = static_cast<const float *>(fl.f[f]);
      const float4 a = *reinterpret_cast<const float4 *>(F + base);
      const float4 c = *reinterpret_cast<const float4 *>(F + base + 4);
      v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = c.x; v[5] = c.y; v[6] = c.z; v[7] = c.w;
    } else {
      const uint16_t *H = static_cast<const uint16_t *>(fl.f[f]);
      const uint4 u = *reinterpret_cast<const uint4 *>(H + base);  // 8 x 16 bit
      const uint32_t w4[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        v[2 * i] = h16_to_f((uint16_t)(w4[i] & 0xFFFFu), fl.mode[f]);
        v[2 * i + 1] = h16_to_f((uint16_t)(w4[i] >> 16), fl.mode[f]);
      }
    }
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 8; i++) acc = acc + v[i];
    const float mean = acc * 0.125f;
    if (fl.mode[f] == 0) static_cast<float *>(fl.f[f])[pc] = mean;
    else static_cast<uint16_t *>(fl.f[f])[pc] = f_to_h16(mean, fl.mode[f]);
  }
}

// k_dcgrid_calc_divergence (dcgrid_fluid.cu:174-230): zero p, p~, div on all
// cells; div on leaf cells from fluidity-weighted central differences, apron
// velocities through the boundary conditions.
__device__ __forceinline__ void divergence_cell(const Dev &D, long long b, int c) {
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const size_t cell = (size_t)b * BV + c;
  D.p[cell] = 0.f;
  D.pt[cell] = 0.f;
  float dv = 0.f;
  if (D.child[cell >> 3] == NONE) {
    int lx, ly, lz;
    local_xyz(c, lx, ly, lz);
    const int ax = lx + 1, ay = ly + 1, az = lz + 1;
    const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz;
    const int scale = 1 << bp.w;
    const float alpha = 0.5f * D.ph.rdx / (float)scale;
    float nbv[6];
    float nbw[6];
    const int off[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
#pragma unroll
    for (int n = 0; n < 6; n++) {
      const int i = ax + off[n][0], j = ay + off[n][1], k = az + off[n][2];
      const unsigned long long nc = apron_cell(D, (uint32_t)b, bp, i, j, k);
      nbw[n] = D.w[nc];
      const int comp = n >> 1;
      float v = D.v[comp][nc];
      if (i == 0 || i == AW - 1 || j == 0 || j == AW - 1 || k == 0 || k == AW - 1)
        v = vel_bc1(D.g, D.ph, v, comp, x + off[n][0], y + off[n][1], z + off[n][2], scale);
      nbv[n] = v;
    }
    dv = alpha * (nbw[1] * nbv[1] - nbw[0] * nbv[0] + nbw[3] * nbv[3] - nbw[2] * nbv[2] +
                  nbw[5] * nbv[5] - nbw[4] * nbv[4]);
  }
  D.div[cell] = dv;
}

// k_dcgrid_jacobi / _inv (dcgrid_multigrid_solver.cu:5-41) over every
// allocated cell of one level (leaf or covered): dst = (sum6 src - a div) / 6.
__global__ void __launch_bounds__(256) k_jacobi(Dev D, int level, const float *__restrict__ src,
                                                float *__restrict__ dst) {
  const long long bl = (long long)blockIdx.x * 4 + (threadIdx.x >> 6);
  if (bl >= D.g.budget[level]) return;
  const long long b = D.g.off[level] + bl;
  const int4 bp = D.pos[b];
  if (bp.w != level) return;
  const int c = threadIdx.x & 63;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  const int s = 1 << level;
  const float alpha = (float)(s * s) * D.ph.dx * D.ph.dx;
  const float pl = src[apron_cell(D, (uint32_t)b, bp, ax - 1, ay, az)];
  const float pr = src[apron_cell(D, (uint32_t)b, bp, ax + 1, ay, az)];
  const float pd = src[apron_cell(D, (uint32_t)b, bp, ax, ay - 1, az)];
  const float pu = src[apron_cell(D, (uint32_t)b, bp, ax, ay + 1, az)];
  const float pb = src[apron_cell(D, (uint32_t)b, bp, ax, ay, az - 1)];
  const float pf = src[apron_cell(D, (uint32_t)b, bp, ax, ay, az + 1)];
  const size_t cell = (size_t)b * BV + c;
  dst[cell] = div6(pl + pr + pd + pu + pb + pf - alpha * D.div[cell]);
}

// k_dcgrid_prolongate (dcgrid_multigrid_solver.cu:43-76): 27/9/3/1 trilinear
// interpolation from the parent block's apron.
__global__ void __launch_bounds__(256) k_prolongate(Dev D, int level) {
  const long long bl = (long long)blockIdx.x * 4 + (threadIdx.x >> 6);
  if (bl >= D.g.budget[level]) return;
  const long long b = D.g.off[level] + bl;
  const int4 bp = D.pos[b];
  if (bp.w != level) return;
  const uint32_t par = D.parent[b];
  if (par == NONE) return;
  const uint32_t pb = par >> 3;
  const int4 pbp = D.pos[pb];
  const int c = threadIdx.x & 63;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz;
  const int ax = 1 + (x / 2) % BW, ay = 1 + (y / 2) % BW, az = 1 + (z / 2) % BW;
  const int i = x % 2 ? 1 : -1, j = y % 2 ? 1 : -1, k = z % 2 ? 1 : -1;
  const float *P = D.p;
  const float p000 = P[apron_cell(D, pb, pbp, ax, ay, az)];
  const float p001 = P[apron_cell(D, pb, pbp, ax, ay, az + k)];
  const float p010 = P[apron_cell(D, pb, pbp, ax, ay + j, az)];
  const float p100 = P[apron_cell(D, pb, pbp, ax + i, ay, az)];
  const float p011 = P[apron_cell(D, pb, pbp, ax, ay + j, az + k)];
  const float p101 = P[apron_cell(D, pb, pbp, ax + i, ay, az + k)];
  const float p110 = P[apron_cell(D, pb, pbp, ax + i, ay + j, az)];
  const float p111 = P[apron_cell(D, pb, pbp, ax + i, ay + j, az + k)];
  D.p[(size_t)b * BV + c] =
      (27.f * p000 + 9.f * (p001 + p010 + p100) + 3.f * (p011 + p101 + p110) + p111) / 64.f;
}

// One cell of k_prolongate, addressed by its global cell index.
__device__ inline void prolong_cell(const Dev &D, long long cell) {
  const uint32_t b = (uint32_t)(cell >> 6);
  const uint32_t par = D.parent[b];
  if (par == NONE) return;
  const int4 bp = D.pos[b];
  const uint32_t pb = par >> 3;
  const int4 pbp = D.pos[pb];
  int lx, ly, lz;
  local_xyz((int)(cell & 63), lx, ly, lz);
  const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz;
  const int ax = 1 + (x / 2) % BW, ay = 1 + (y / 2) % BW, az = 1 + (z / 2) % BW;
  const int i = x % 2 ? 1 : -1, j = y % 2 ? 1 : -1, k = z % 2 ? 1 : -1;
  const float *P = D.p;
  const float p000 = P[apron_cell(D, pb, pbp, ax, ay, az)];
  const float p001 = P[apron_cell(D, pb, pbp, ax, ay, az + k)];
  const float p010 = P[apron_cell(D, pb, pbp, ax, ay + j, az)];
  const float p100 = P[apron_cell(D, pb, pbp, ax + i, ay, az)];
  const float p011 = P[apron_cell(D, pb, pbp, ax, ay + j, az + k)];
  const float p101 = P[apron_cell(D, pb, pbp, ax + i, ay, az + k)];
  const float p110 = P[apron_cell(D, pb, pbp, ax + i, ay + j, az)];
  const float p111 = P[apron_cell(D, pb, pbp, ax + i, ay + j, az + k)];
  D.p[cell] = (27.f * p000 + 9.f * (p001 + p010 + p100) + 3.f * (p011 + p101 + p110) + p111) / 64.f;
}

// Loads go through L2 (__ldcg): inside one persistent launch the ping-pong
// buffers are rewritten by other SMs, so no SM may serve them from its L1.
__device__ inline float jacobi_update(const float *src, const Nb6 &n, float ad) {
  return div6(__ldcg(src + n.i0) + __ldcg(src + n.i1) + __ldcg(src + n.i2) + __ldcg(src + n.i3) +
              __ldcg(src + n.i4) + __ldcg(src + n.i5) - ad);
}

__device__ inline uint32_t ld_acquire_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline void st_release_u32(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Neighbour epochs: epoch[b] = sweeps block b has completed in the current
// level solve. Before sweep k (1-based) of a CTA's blocks, their same-level
// face neighbours must have completed sweep k-1: then the values read are
// current and nobody still reads the buffer being written. Coarser neighbours
// are constant during the solve and need no wait. Thread i < 24*rounds polls
// face i%6 of block i/6 of the CTA; the wait is bounded (2^22 polls) and
// records DCG_DEVERR_TIMEOUT (8) when exceeded. Writes are ordered before the
// release store by bar.sync; the acquire load orders later reads the same way.
__device__ inline long long cta_block(long long off, int j, unsigned nctas) {
  return off + 4 * ((long long)(j >> 2) * nctas + blockIdx.x) + (j & 3);
}
__device__ inline void wait_neighbours(const Dev &D, long long off, long long blk_end, int rounds, unsigned nctas,
                                       uint32_t need) {
  const int t = threadIdx.x;
  if (need > 0 && t < 24 * rounds) {
    const long long b = cta_block(off, t / 6, nctas);
    if (b < blk_end) {
      const int f = t % 6;
      const int dir = f == 0 ? 4 : f == 1 ? 22 : f == 2 ? 10 : f == 3 ? 16 : f == 4 ? 12 : 14;
      const uint32_t e = D.nbr[27 * b + dir];
      if (e != OUT && (e >> 28) == 0 && (e & NBR_MASK) != (uint32_t)b) {
        const uint32_t *ep = D.epoch + (e & NBR_MASK);
        unsigned spins = 0;
        while (ld_acquire_u32(ep) < need) {
          if (++spins > (1u << 22) || (*(volatile uint32_t *)D.err & 8u)) {
            atomicOr(D.err, 8u);
            break;
          }
          __nanosleep(20);
        }
      }
    }
  }
  __syncthreads();
}
__device__ inline void publish_blocks(const Dev &D, long long off, long long blk_end, int rounds, unsigned nctas,
                                      uint32_t done) {
  __syncthreads();
  const int t = threadIdx.x;
  if (t < 4 * rounds) {
    const long long b = cta_block(off, t, nctas);
    if (b < blk_end) st_release_u32(D.epoch + b, done);
  }
}

constexpr int LS_CACHE = 4;

// The solve of one level of the cascade (fluid_simulation_dcgrid.cu:281-290)
// in one cooperative launch: optional prolongation from the parent level, then
// `sweeps` Jacobi sweeps (ping-pong p -> p~ -> p, as k_dcgrid_jacobi/_inv).
// Work split: CTA c owns the level's blocks 4*(r*grid + c) .. +3 in round r.
// One grid barrier follows prolongation and the epoch reset; sweeps are then
// separated by a flat (epoch_sync 0) or two-level (2) grid barrier, or ordered
// block by block through neighbour epochs (1). The library uses this kernel
// only where the staged solve (k_level_solve_batch) cannot form its
// cooperative grid, with the two-level barrier.
// The level's topology is fixed during the solve, so each thread resolves the
// six neighbour cells of its (at most LS_CACHE) cells once and keeps them and
// alpha*div in registers; a sweep is then six loads and one store per cell.
// Levels with more cells than the grid covers in LS_CACHE rounds resolve
// neighbours in every sweep. Arithmetic is that of k_jacobi (identical results).
template <int CACHE>
__global__ void __launch_bounds__(256) k_level_solve(Dev D, int level, int prolong, int sweeps, int epoch_sync) {
  const unsigned nctas = gridDim.x;
  const long long nblk = D.load[level];
  const long long ncell = nblk * 64;
  const long long off = D.g.off[level];
  const long long base = off * 64;
  const long long stride = (long long)nctas * 256;
  const long long first = (long long)blockIdx.x * 256 + threadIdx.x;
  const int rounds = (int)((ncell + stride - 1) / stride);
  const int s = 1 << level;
  const float alpha = (float)(s * s) * D.ph.dx * D.ph.dx;
  for (long long b = first; b < nblk; b += stride) D.epoch[off + b] = 0u;
  if (prolong)
    for (long long lc = first; lc < ncell; lc += stride) prolong_cell(D, base + lc);
  if (sweeps <= 0) return;
  // epoch_sync: 0 = flat grid barrier, 1 = neighbour epochs, 2 = two-level barrier
  auto barrier = [&]() {
    if (epoch_sync == 2) grid_barrier_tree(D, nctas);
    else grid_barrier(D, nctas);
  };
  barrier();
  const long long blk_end = off + nblk;
  if (CACHE > 0 && rounds <= CACHE) {
    // neighbour indices and alpha*div of the thread's cells, [round][k][thread]
    __shared__ uint32_t s_nb[CACHE > 0 ? CACHE : 1][6][256];
    __shared__ float s_ad[CACHE > 0 ? CACHE : 1][256];
    const int t = threadIdx.x;
    for (int r = 0; r < rounds; r++) {
      const long long lc = first + r * stride;
      if (lc < ncell) {
        const Nb6 n = jacobi_neighbours(D, base + lc);
        s_nb[r][0][t] = n.i0; s_nb[r][1][t] = n.i1; s_nb[r][2][t] = n.i2;
        s_nb[r][3][t] = n.i3; s_nb[r][4][t] = n.i4; s_nb[r][5][t] = n.i5;
        s_ad[r][t] = alpha * D.div[base + lc];
      }
    }
    for (int it = 0; it < sweeps; it++) {
      const float *src = (it & 1) ? D.pt : D.p;
      float *dst = (it & 1) ? D.p : D.pt;
      if (epoch_sync == 1) wait_neighbours(D, off, blk_end, rounds, nctas, (uint32_t)it);
      for (int r = 0; r < rounds; r++) {
        const long long lc = first + r * stride;
        if (lc < ncell) {
          const Nb6 n = {s_nb[r][0][t], s_nb[r][1][t], s_nb[r][2][t], s_nb[r][3][t], s_nb[r][4][t], s_nb[r][5][t]};
          dst[base + lc] = jacobi_update(src, n, s_ad[r][t]);
        }
      }
      if (epoch_sync == 1) publish_blocks(D, off, blk_end, rounds, nctas, (uint32_t)it + 1);
      else if (it + 1 < sweeps) barrier();
    }
  } else {
    // too many rounds for the caches: neighbours resolved every sweep, and a
    // grid barrier between sweeps (epochs would need 24 pollers per block)
    for (int it = 0; it < sweeps; it++) {
      const float *src = (it & 1) ? D.pt : D.p;
      float *dst = (it & 1) ? D.p : D.pt;
      for (long long lc = first; lc < ncell; lc += stride)
        dst[base + lc] = jacobi_update(src, jacobi_neighbours(D, base + lc), alpha * D.div[base + lc]);
      if (it + 1 < sweeps) barrier();
    }
  }
}

// k_dcgrid_apply_pressure (dcgrid_fluid.cu:232-259) on leaf cells.
__device__ __forceinline__ void apply_pressure_cell(const Dev &D, long long b, int c) {
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  const int scale = 1 << bp.w;
  const float alpha = 0.5f * D.ph.rdx / (float)scale;
  const float pc = D.p[cell];
  const unsigned long long L = apron_cell(D, (uint32_t)b, bp, ax - 1, ay, az);
  const unsigned long long R = apron_cell(D, (uint32_t)b, bp, ax + 1, ay, az);
  const unsigned long long Dn = apron_cell(D, (uint32_t)b, bp, ax, ay - 1, az);
  const unsigned long long U = apron_cell(D, (uint32_t)b, bp, ax, ay + 1, az);
  const unsigned long long Bk = apron_cell(D, (uint32_t)b, bp, ax, ay, az - 1);
  const unsigned long long F = apron_cell(D, (uint32_t)b, bp, ax, ay, az + 1);
  const float *P = D.p, *W = D.w;
  D.v[0][cell] = D.v[0][cell] - alpha * (W[R] * (P[R] - pc) + W[L] * (pc - P[L]));
  D.v[1][cell] = D.v[1][cell] - alpha * (W[U] * (P[U] - pc) + W[Dn] * (pc - P[Dn]));
  D.v[2][cell] = D.v[2][cell] - alpha * (W[F] * (P[F] - pc) + W[Bk] * (pc - P[Bk]));
}

// ---------------------------------------------------------------- defect correction
// The FP64 residual of every allocated cell's Jacobi equation is cell stage 6
// of k_cells_staged.
// p += e on every allocated cell
__device__ __forceinline__ void add_correction_cell(const Dev &D, long long b) {
  if (b >= D.g.B || D.pos[b].w < 0) return;
  const long long cell = b * BV + (threadIdx.x & 63);
  D.p[cell] = D.p[cell] + D.e[cell];
}
__global__ void __launch_bounds__(256) k_add_correction(Dev D) {
  add_correction_cell(D, (long long)blockIdx.x * 4 + (threadIdx.x >> 6));
}

// ------------------------------------------------------------ single-simulation kernels
// 256-thread CTAs, 4 blocks of 64 cells per CTA.
__device__ __forceinline__ long long cta_block4() { return (long long)blockIdx.x * 4 + (threadIdx.x >> 6); }
__global__ void __launch_bounds__(256) k_advect_velocity(Dev D) { advect_velocity_cell(D, cta_block4(), threadIdx.x & 63); }
__global__ void __launch_bounds__(256) k_advect_scalars(Dev D) { advect_scalars_cell(D, cta_block4(), threadIdx.x & 63); }
__global__ void __launch_bounds__(256) k_divergence(Dev D) { divergence_cell(D, cta_block4(), threadIdx.x & 63); }
__global__ void __launch_bounds__(256) k_apply_pressure(Dev D) { apply_pressure_cell(D, cta_block4(), threadIdx.x & 63); }
__global__ void __launch_bounds__(256) k_restrict(Dev D, int level, FieldList fl) {
  restrict_subblock(D, level, fl, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------------------------------ launchers
static inline unsigned cta_blocks(long long nblocks) { return (unsigned)((nblocks + 3) / 4); }

void launch_advect_velocity(const Dev &D, cudaStream_t st) {
  k_advect_velocity<<<cta_blocks(D.g.B), 256, 0, st>>>(D);
}
void launch_advect_scalars(const Dev &D, cudaStream_t st) {
  k_advect_scalars<<<cta_blocks(D.g.B), 256, 0, st>>>(D);
}
void launch_sources(const Dev &D, cudaStream_t st) { k_sources<<<cta_blocks(D.g.B), 256, 0, st>>>(D); }
void launch_add_noise(const Dev &D, unsigned long long seed, float amp, cudaStream_t st) {
  k_add_noise<<<cta_blocks(D.g.B), 256, 0, st>>>(D, seed, amp);
}
void launch_restrict(const Dev &D, const FieldList &fl, cudaStream_t st) {
  for (int level = 0; level < D.g.levels - 1; level++) {
    const long long n = 8 * D.g.budget[level];
    k_restrict<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(D, level, fl);
  }
}
void launch_divergence(const Dev &D, cudaStream_t st) { k_divergence<<<cta_blocks(D.g.B), 256, 0, st>>>(D); }
void launch_jacobi(const Dev &D, int level, const float *src, float *dst, cudaStream_t st) {
  k_jacobi<<<cta_blocks(D.g.budget[level]), 256, 0, st>>>(D, level, src, dst);
}
void launch_prolongate(const Dev &D, int level, cudaStream_t st) {
  k_prolongate<<<cta_blocks(D.g.budget[level]), 256, 0, st>>>(D, level);
}
void launch_add_correction(const Dev &D, cudaStream_t st) { k_add_correction<<<cta_blocks(D.g.B), 256, 0, st>>>(D); }
void launch_apply_pressure(const Dev &D, cudaStream_t st) {
  k_apply_pressure<<<cta_blocks(D.g.B), 256, 0, st>>>(D);
}
// Both variants are launched with the grid of the cached one (the smaller
// per-SM occupancy), so either fits co-resident.
int level_solve_grid(int sms) {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_level_solve<LS_CACHE>, 256, 0) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_level_solve<0>, 256, 0) != cudaSuccess) return 0;
  return (a < b ? a : b) * sms;
}
void launch_level_solve(const Dev &D, int level, int prolong, int sweeps, int grid, int epoch_sync, cudaStream_t st) {
  // cells of the level are known only on the device; the cached variant
  // falls back to per-sweep neighbour resolution when they exceed its rounds,
  // and the uncached variant serves budgets that cannot fit at all.
  const long long max_cells = D.g.budget[level] * 64;
  const bool cached = max_cells <= (long long)grid * 256 * LS_CACHE * 4;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cached) cudaLaunchKernelEx(&cfg, k_level_solve<LS_CACHE>, D, level, prolong, sweeps, epoch_sync);
  else cudaLaunchKernelEx(&cfg, k_level_solve<0>, D, level, prolong, sweeps, epoch_sync == 2 ? 2 : 0);
}

// ------------------------------------------------------------------ batched kernels
// Many independent simulations per launch. CTA ranges are assigned to the
// members in order (P.end is cumulative); a CTA finds its member with a short
// scan of uniform parameter loads and runs the same cell body as the
// single-simulation kernels, so a member's results are bit-identical to those
// of a standalone simulation. TB = blocks of 64 cells per CTA (the tile).
__device__ __forceinline__ int batch_member(const long long *end, int n, long long x) {
  int s = 0;
  while (s + 1 < n && x >= end[s]) s++;
  return s;
}

template <int TB, int STAGE>
__global__ void __launch_bounds__(64 * TB) k_cells_batch(const __grid_constant__ CellBatch P) {
  const int s = batch_member(P.end, P.n, blockIdx.x);
  const long long b = ((long long)blockIdx.x - (s ? P.end[s - 1] : 0)) * TB + (threadIdx.x >> 6);
  const Dev &D = P.d[s];
  const int c = threadIdx.x & 63;
  if (STAGE == 0) advect_velocity_cell(D, b, c);
  else if (STAGE == 1) advect_scalars_cell(D, b, c);
  else if (STAGE == 2) divergence_cell(D, b, c);
  else if (STAGE == 3) apply_pressure_cell(D, b, c);
  else stats_cell(D, b, c);
}

// Persistent form: a grid of a few CTAs per SM walks only the allocated
// blocks. Segment (member m, level l) holds ceil(load_m[l] / TB) tiles of TB
// blocks starting at off_m[l]; every CTA builds the cumulative tile counts in
// shared memory from the device-side loads, then takes tiles blockIdx.x,
// blockIdx.x + gridDim.x, ...
template <int TB, int STAGE>
__global__ void __launch_bounds__(64 * TB) k_cells_persist(const __grid_constant__ CellBatch P) {
  __shared__ long long s_end[BMAX * MAXL];
  __shared__ long long s_cnt[BMAX * MAXL];
  const int nseg = P.n * MAXL;
  for (int i = threadIdx.x; i < nseg; i += blockDim.x) {
    const Dev &D = P.d[i / MAXL];
    const int l = i % MAXL;
    const long long cnt = l < D.g.levels ? __ldcg(D.load + l) : 0;
    s_cnt[i] = cnt;
    s_end[i] = (cnt + TB - 1) / TB;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 1; i < nseg; i++) s_end[i] += s_end[i - 1];
  __syncthreads();
  const long long total = s_end[nseg - 1];
  const int c = threadIdx.x & 63;
  // statistics: every thread sums its cells' values in FP64 registers while
  // the warp's member and level stay the same; a change (and the end) reduces
  // the warp's sums and adds them with one atomic per quantity
  double a_res = 0.0, a_mass = 0.0;
  int a_cnt = 0, a_mem = -1, a_lvl = 0;
  auto flush = [&]() {
    double r = a_res, m = a_mass;
    for (int o = 16; o > 0; o >>= 1) {
      r += __shfl_xor_sync(0xffffffffu, r, o);
      m += __shfl_xor_sync(0xffffffffu, m, o);
    }
    const int n = (int)__reduce_add_sync(0xffffffffu, (unsigned)a_cnt);
    stats_flush(P.d[a_mem], r, m, a_lvl, (double)n);
  };

  for (long long t = blockIdx.x; t < total; t += gridDim.x) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (t < s_end[mid]) hi = mid;
      else lo = mid + 1;
    }
    const Dev &D = P.d[lo / MAXL];
    const int l = lo % MAXL;
    const long long k = (t - (lo ? s_end[lo - 1] : 0)) * TB + (threadIdx.x >> 6);
    // out-of-segment lanes get b = B: every body returns there (the statistics
    // body still joins its warp reductions)
    const long long b = k < s_cnt[lo] ? D.g.off[l] + k : D.g.B;
    if (STAGE == 0) advect_velocity_cell(D, b, c);
    else if (STAGE == 1) advect_scalars_cell(D, b, c);
    else if (STAGE == 2) divergence_cell(D, b, c);
    else if (STAGE == 3) apply_pressure_cell(D, b, c);
    else {
      float r, m;
      const int lev = stats_vals(D, b, c, r, m);
      const unsigned leaf = __ballot_sync(0xffffffffu, lev >= 0);
      if (leaf) {  // warp-uniform: a warp covers half of one block
        const int lvl = __shfl_sync(0xffffffffu, lev, __ffs(leaf) - 1);
        const int mem = lo / MAXL;
        if (mem != a_mem || lvl != a_lvl) {
          if (a_mem >= 0) flush();
          a_mem = mem;
          a_lvl = lvl;
          a_res = a_mass = 0.0;
          a_cnt = 0;
        }
        a_res += (double)r;
        a_mass += (double)m;
        a_cnt += lev >= 0;
      }
    }
  }
  if (STAGE == 4 && a_mem >= 0) flush();
}

__global__ void __launch_bounds__(128) k_stats_zero(const __grid_constant__ CellBatch P) {
  if (threadIdx.x < 32) P.d[blockIdx.x].red[threadIdx.x] = 0.0;
}
__global__ void __launch_bounds__(128) k_stats_gather(const __grid_constant__ CellBatch P, StatRecord *dst) {
  const Dev &D = P.d[blockIdx.x];
  StatRecord &r = dst[blockIdx.x];
  const int t = threadIdx.x;
  if (t < 32) r.red[t] = __ldcg(D.red + t);
  if (t < C_COUNT) r.ctr[t] = __ldcg(D.ctr + t);
  if (t < MAXL) r.load[t] = __ldcg(D.load + t);
  if (t == 0) r.err = __ldcg(D.err);
  // defect correction: the norms before the first and after the last pass
  if (t < 4) r.dn[t] = D.g.dpass > 0 ? __ldcg(D.dnorm + (t < 2 ? t : 2 * D.g.dpass + t - 2)) : 0.0;
}
void launch_stats_zero(const CellBatch &P, cudaStream_t st) { k_stats_zero<<<P.n, 128, 0, st>>>(P); }
void launch_stats_gather(const CellBatch &P, StatRecord *dst, cudaStream_t st) {
  k_stats_gather<<<P.n, 128, 0, st>>>(P, dst);
}

// p += e on every allocated cell of every member of a batch (4 blocks per
// CTA, P.end cumulative); the cell body is the single simulation's.
__global__ void __launch_bounds__(256) k_add_correction_batch(const __grid_constant__ CellBatch P) {
  const int s = batch_member(P.end, P.n, blockIdx.x);
  add_correction_cell(P.d[s], ((long long)blockIdx.x - (s ? P.end[s - 1] : 0)) * 4 + (threadIdx.x >> 6));
}
void launch_add_correction_batch(CellBatch &P, cudaStream_t st) {
  long long acc = 0;
  for (int m = 0; m < P.n; m++) {
    acc += (P.d[m].g.B + 3) / 4;
    P.end[m] = acc;
  }
  if (acc > 0) k_add_correction_batch<<<(unsigned)acc, 256, 0, st>>>(P);
}

__global__ void __launch_bounds__(256) k_restrict_batch(const __grid_constant__ RestrictBatch P) {
  const int s = batch_member(P.end, P.n, blockIdx.x);
  const Dev &D = P.d[s];
  if (P.level >= D.g.levels - 1) return;
  restrict_subblock(D, P.level, P.fl[s], ((long long)blockIdx.x - (s ? P.end[s - 1] : 0)) * 256 + threadIdx.x);
}

// Description of one block for the staged sweep, BI_WORDS words: [BI_OWN]
// arena index of its first cell, [BI_ALPHA] alpha (bits), [BI_CODES..+1] one
// byte per face (-x, +x, -y, +y, -z, +z): levels by which the block that holds
// the face's halo is coarser, 16 for outside, 17 for outside under the compat
// quirk of apron_cell, [BI_FACE..+5] arena index of the first cell of that
// block (the block itself when the face is outside), [BI_POS..+2] level-local
// position, the rest zero. 16 words, so that a lane reads words 0-3 and 4-7
// with one 16-byte load each and faces 4-5 with one 8-byte load. Lanes 0-5
// resolve one face each, lane 6 the rest.
__device__ __forceinline__ void fill_block_info(const SolveBatch &P, const long long *s_end, const int *s_lev,
                                                long long gb, uint32_t *bi, int lane) {
  const int m = batch_member(s_end, P.n, gb << 6);
  const Dev &D = P.d[m];
  const int lev = s_lev[m];
  const uint32_t b = (uint32_t)(D.g.off[lev] + (gb - (m ? (s_end[m - 1] >> 6) : 0)));
  const uint32_t a = (uint32_t)P.arena[m];
  if (lane < 6) {
    const int dir = lane == 0 ? 4 : lane == 1 ? 22 : lane == 2 ? 10 : lane == 3 ? 16 : lane == 4 ? 12 : 14;
    const uint32_t e = D.nbr[27u * b + dir];
    uint32_t base, code;
    if (e == OUT) {
      base = a + b * BV;
      code = (D.g.ref_compat && lev < D.g.sparse) ? 17u : 16u;
    } else {
      base = a + (e & NBR_MASK) * BV;
      code = e >> 28;
    }
    bi[BI_FACE + lane] = base;
    reinterpret_cast<uint8_t *>(bi + BI_CODES)[lane] = (uint8_t)code;
  } else if (lane == 6) {
    const int4 bp = D.pos[b];
    bi[BI_OWN] = a + b * BV;
    const int sc = 1 << lev;
    bi[BI_ALPHA] = __float_as_uint((float)(sc * sc) * D.ph.dx * D.ph.dx);
    bi[BI_POS] = (uint32_t)bp.x;
    bi[BI_POS + 1] = (uint32_t)bp.y;
    bi[BI_POS + 2] = (uint32_t)bp.z;
    for (int j = BI_POS + 3; j < BI_WORDS; j++) bi[j] = 0u;
  }
}

// Staged-sweep schedule: blocks per warp pass, software pipelining of the
// next pass's loads, and the minimum resident CTAs per SM the register
// allocation targets.
#ifndef DCG_SOLVE_U
#define DCG_SOLVE_U 2
#endif
#ifndef DCG_SOLVE_PIPE
#define DCG_SOLVE_PIPE 0
#endif
#ifndef DCG_SOLVE_MINB
#define DCG_SOLVE_MINB 4
#endif
#ifndef DCG_PIPE_MINB
#define DCG_PIPE_MINB 3
#endif
#ifndef DCG_PIPE_CLAIM
#define DCG_PIPE_CLAIM 2
#endif

// ---- pipelined staged sweeps
// Asynchronous copies (cp.async, Ampere+ LDGSTS) of 4 and 8 bytes from global
// memory into shared memory: the data goes to the tile without passing
// through registers, so a warp keeps the loads of the next NB-1 blocks in
// flight while it computes the current one.
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}
// the same with a 32-bit shared-memory address
__device__ __forceinline__ void cp_async4s(uint32_t dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8s(uint32_t dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Staged sweeps as in the per-pass form below, pipelined: the warps of a CTA
// claim the CTA's blocks (level blocks ((r * nctas + blockIdx.x) * 8 + w'))
// from a shared counter, so faster warps take more of them, and each warp
// cycles its blocks through NB tile buffers: the copies of its next NB - 1
// blocks (own cells, three halo cells per lane, divergence) are in flight
// while a block is computed from its tile.
// The copies read the previous sweep's results written by other SMs; the grid
// barrier's fences order them. Block descriptions come from the launch's
// shared cache when they fit, else from the global table: every lane loads
// the words it needs (warp-wide broadcasts). Broadcast loads cost the
// shared-memory pipe, which bounds the sweep, less than warp shuffles of the
// same words do; measured on the 16-plume batch, so are the shuffles that
// would replace the tile reads of the neighbours inside the block.
template <int CACHE, int NB, int CLAIM>
__device__ __forceinline__ void solve_pipelined(const SolveBatch &P, const long long *s_end, const int *s_lev,
                                                uint32_t *s_cache, long long total, unsigned nctas, int sweeps,
                                                int tree) {
  constexpr int W = 8, SX = DCG_TILE_SX, SY = DCG_TILE_SY, TILE = 5 * SX + 5 * SY + 8;
  __shared__ __align__(16) float s_pt[W][NB][TILE];
  __shared__ __align__(16) float s_pd[W][NB][64];
  const unsigned full = 0xffffffffu;
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  int oA;
  uint32_t hpk[3], hax[3];
  halo_slots<SX, SY>(lane, oA, hpk, hax);
  const long long nblocks = total >> 6;
  const int rounds_b = (int)((nblocks + (long long)W * nctas - 1) / ((long long)W * nctas));
  const bool cached = rounds_b <= CACHE * 2048 / (W * BI_WORDS);
  for (int r = 0; r < rounds_b; r++) {
    const long long gb = ((long long)r * nctas + blockIdx.x) * W + w;
    if (gb >= nblocks) continue;
    if (cached) {
      fill_block_info(P, s_end, s_lev, gb, s_cache + (r * W + w) * BI_WORDS, lane);
    } else {
      __shared__ uint32_t s_one[W][BI_WORDS];
      fill_block_info(P, s_end, s_lev, gb, s_one[w], lane);
      __syncwarp();
      if (lane < BI_WORDS) P.binfo[gb * BI_WORDS + lane] = s_one[w][lane];
      __syncwarp();
    }
  }
  // blocks are claimed dynamically inside the CTA: CTA-local block k = r * W +
  // w' is level block ((r * nctas + blockIdx.x) * W + w'), valid for k < kcount
  __shared__ unsigned s_next[2];
  if (t == 0) s_next[0] = s_next[1] = 0u;
  __syncthreads();  // block descriptions filled by every warp, counters zeroed
  int kcount = 0;
  for (int r = 0; r < rounds_b; r++) {
    const long long g0 = ((long long)r * nctas + blockIdx.x) * W;
    const long long left = nblocks - g0;
    kcount += left <= 0 ? 0 : (left >= W ? W : (int)left);
  }
  auto barrier = [&]() {
    if (tree & 1) grid_barrier_tree(P.bar, P.err, nctas);
    else grid_barrier(P.bar, P.err, nctas);
  };
  // per buffer: arena index of the block's first cell and alpha (bits); own = ~0u: no block
  uint32_t b_own[NB], b_alpha[NB];
  // shared-memory addresses of the lane's copy targets in buffer 0 (buffer b: + b * TILE * 4)
  const uint32_t s_own = (uint32_t)__cvta_generic_to_shared(&s_pt[w][0][oA]);
  uint32_t s_halo[3];
#pragma unroll
  for (int q = 0; q < 3; q++) s_halo[q] = (uint32_t)__cvta_generic_to_shared(&s_pt[w][0][hpk[q] & 511u]);
  const uint32_t s_div = (uint32_t)__cvta_generic_to_shared(&s_pd[w][0][2 * lane]);
  const float *divl = P.div + 2 * lane;
  for (int it = 0; it < sweeps; it++) {
    const float *src = (it & 1) ? P.pt : P.p;
    float *dst = (it & 1) ? P.p : P.pt;
    const float *srcl = src + 2 * lane;
    float2 *dstl = reinterpret_cast<float2 *>(dst) + lane;
    if (t == 0) s_next[(it + 1) & 1] = 0u;  // the next sweep's counter; its last use ended before the barrier
    unsigned *cnt = &s_next[it & 1];
    // a warp claims CLAIM consecutive CTA-local blocks per counter update
    // (fewer shared atomics and broadcasts per block; on the batch's large
    // rounds two measured best, 3, 4 and 8 balance the warps worse; one for
    // levels of a few blocks per warp, which the pairs would unbalance)
    int kpend = 0, npend = 0;
    auto issue = [&](int buf) {
      int k;
      if (CLAIM > 1 && npend > 0) {
        k = kpend++;
        npend--;
      } else {
        unsigned kk = 0;
        if (lane == 0) kk = atomicAdd(cnt, (unsigned)CLAIM);
        k = (int)__shfl_sync(full, kk, 0);
        kpend = k + 1;
        npend = CLAIM - 1;
      }
      const bool act = k < kcount;  // warp-uniform; a warp's claims only grow
      // the block's description: words 0-9 in three warp-wide broadcast
      // loads (16, 16 and 8 bytes) from the launch's shared cache or the
      // global table; a lane's halo slot q lies on face 2q or 2q + 1
      static_assert(BI_OWN == 0 && BI_ALPHA == 1 && BI_CODES == 2 && BI_FACE == 4 && BI_WORDS % 4 == 0,
                    "description words read as (own, alpha, codes), faces 0-3, faces 4-5");
      const long long gbk = ((long long)(k >> 3) * nctas + blockIdx.x) * W + (k & 7);
      const uint32_t *big = P.binfo + gbk * BI_WORDS, *bis = s_cache + k * BI_WORDS;
      uint4 wa = make_uint4(0u, 0u, 0u, 0u), wb = make_uint4(0u, 0u, 0u, 0u);
      uint2 wc = make_uint2(0u, 0u);
      if (act) {
        if (cached) {
          wa = *reinterpret_cast<const uint4 *>(bis);
          wb = *reinterpret_cast<const uint4 *>(bis + 4);
          wc = *reinterpret_cast<const uint2 *>(bis + 8);
        } else {
          wa = __ldcg(reinterpret_cast<const uint4 *>(big));
          wb = __ldcg(reinterpret_cast<const uint4 *>(big + 4));
          wc = __ldcg(reinterpret_cast<const uint2 *>(big + 8));
        }
      }
      const uint32_t own = wa.x, alpha = wa.y, c11 = wa.z, c12 = wa.w;
      const uint32_t fb[3] = {((hax[0] >> 12) & 1u) ? wb.y : wb.x, ((hax[1] >> 12) & 1u) ? wb.w : wb.z,
                              ((hax[2] >> 12) & 1u) ? wc.y : wc.x};
      uint32_t addr[3];
      if (c11 == 0u && (c12 & 0xFFFFu) == 0u) {  // all six faces border same-level blocks
#pragma unroll
        for (int q = 0; q < 3; q++) addr[q] = fb[q] + ((hpk[q] >> 9) & 63u);
      } else {
        const uint32_t *bip = (cached ? bis : big) + BI_POS;
        const int bx = (int)(cached ? bip[0] : __ldcg(bip)), by = (int)(cached ? bip[1] : __ldcg(bip + 1)),
                  bz = (int)(cached ? bip[2] : __ldcg(bip + 2));
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const uint32_t pk = hpk[q], ga = hax[q];
          const int f = (int)(ga >> 12);
          const int code = (int)(((f < 4 ? c11 : c12) >> (8 * (f & 3))) & 0xFFu);
          uint32_t li = code == 0 ? (pk >> 9) & 63u : code == 16 ? (pk >> 15) & 63u : (pk >> 21) & 63u;
          if (code > 0 && code < 16) {  // coarser by `code` levels: injection
            const int cx = bx + (int)(ga & 15u) - 1, cy = by + (int)((ga >> 4) & 15u) - 1,
                      cz = bz + (int)((ga >> 8) & 15u) - 1;
            li = (uint32_t)local_of((cx >> code) & 3, (cy >> code) & 3, (cz >> code) & 3);
          }
          addr[q] = fb[q] + li;
        }
      }
      b_own[buf] = act ? own : ~0u;
      b_alpha[buf] = alpha;
      if (act) {
        const uint32_t bo = (uint32_t)(buf * TILE * 4);
        cp_async8s(s_own + bo, srcl + own);
#pragma unroll
        for (int q = 0; q < 3; q++) cp_async4s(s_halo[q] + bo, src + addr[q]);
        cp_async8s(s_div + (uint32_t)(buf * 64 * 4), divl + own);
      }
      cp_async_commit();
    };
#pragma unroll
    for (int k = 0; k < NB - 1; k++) issue(k);
    bool done = false;
    while (!done)
#pragma unroll
    for (int buf = 0; buf < NB; buf++) {  // the warp's blocks cycle through the buffers in claim order
      if (done) break;
      issue((buf + NB - 1) % NB);
      cp_async_wait<NB - 1>();  // the copies of the block in `buf` are complete
      __syncwarp();
      const uint32_t own = b_own[buf];
      done = own == ~0u;  // no block claimed: every later claim of this warp is empty too
      if (own != ~0u) {
        const float *T = s_pt[w][buf];
        const float2 ab = *reinterpret_cast<const float2 *>(T + oA);
        const float2 L = *reinterpret_cast<const float2 *>(T + oA - SX);
        const float2 R = *reinterpret_cast<const float2 *>(T + oA + SX);
        const float2 Dn = *reinterpret_cast<const float2 *>(T + oA - SY);
        const float2 Up = *reinterpret_cast<const float2 *>(T + oA + SY);
        const float Bk = T[oA - 1], Fw = T[oA + 2];
        const float2 dv = *reinterpret_cast<const float2 *>(s_pd[w][buf] + 2 * lane);
        const float al = __uint_as_float(b_alpha[buf]);
        // the lane's two cells with packed FP32x2 operations, each component
        // the correctly rounded operation of the scalar form in the same order:
        // cell a: L + R + D + U + B + (cell b) - alpha div; cell b: L + R + D +
        // U + (cell a) + F - alpha div
        float2 sum = __fadd2_rn(L, R);
        sum = __fadd2_rn(sum, Dn);
        sum = __fadd2_rn(sum, Up);
        sum = __fadd2_rn(sum, make_float2(Bk, ab.x));
        sum = __fadd2_rn(sum, make_float2(ab.y, Fw));
        const float2 ad = __fmul2_rn(make_float2(al, al), dv);
        sum = __fadd2_rn(sum, make_float2(-ad.x, -ad.y));
        dstl[own >> 1] = div6x2(sum);
      }
      __syncwarp();  // buffer `buf` may be refilled by the next issue
    }
    cp_async_wait<0>();
    if (it + 1 < sweeps) barrier();
  }
}

// One round of the batched cascade: level maxtop - round of every member that
// has it, optional prolongation from the member's parent level, then `sweeps`
// Jacobi sweeps over the concatenated cells of all members, separated by grid
// barriers (tree & 1: two-level barrier). Member m's cells of the level
// occupy [s_end[m-1], s_end[m]) of the concatenated index. With CACHE > 0 and
// at most CACHE cells per thread, each thread keeps, per cell, the six
// neighbour cells and its own cell as arena indices plus alpha*div in dynamic
// shared memory ([CACHE][8][256] words); a sweep is then six loads and one
// store per cell. Larger levels are swept one block per warp through a 6^3
// shared-memory tile holding the block and its face halo. Arithmetic is that
// of k_jacobi (identical results).
template <int CACHE, int NB = 0, int MB = DCG_PIPE_MINB, int CLAIM = DCG_PIPE_CLAIM>
__global__ void __launch_bounds__(256, NB ? MB : DCG_SOLVE_MINB)
    k_level_solve_batch(const __grid_constant__ SolveBatch P, int round, int sweeps, int tree) {
  __shared__ long long s_end[BMAX];
  __shared__ int s_lev[BMAX];
  extern __shared__ __align__(16) uint32_t s_cache[];
  const int t = threadIdx.x;
  if (t == 0) {
    long long acc = 0;
    for (int m = 0; m < P.n; m++) {
      const Dev &D = P.d[m];
      // rounds aligned at every member's finest level (round r: level maxtop - r)
      // or, with tree & 2, at its coarsest (round r: level levels - 1 - r)
      const int lev = (tree & 2) ? D.g.levels - 1 - round : P.maxtop - round;
      if (lev >= 0 && lev < D.g.levels) acc += __ldcg(D.load + lev) * 64;
      s_lev[m] = lev;
      s_end[m] = acc;
    }
  }
  __syncthreads();
  const long long total = s_end[P.n - 1];
  const unsigned nctas = gridDim.x;
  const long long stride = (long long)nctas * 256;
  const long long first = (long long)blockIdx.x * 256 + t;
  auto cell_of = [&](long long gi, int &m) {
    m = batch_member(s_end, P.n, gi);
    return P.d[m].g.off[s_lev[m]] * 64 + (gi - (m ? s_end[m - 1] : 0));
  };
  if (P.prolong)
    for (long long gi = first; gi < total; gi += stride) {
      int m;
      const long long cell = cell_of(gi, m);
      if (s_lev[m] < P.d[m].g.levels - 1) prolong_cell(P.d[m], cell);
    }
  if (sweeps <= 0) return;
  auto barrier = [&]() {
    if (tree & 1) grid_barrier_tree(P.bar, P.err, nctas);
    else grid_barrier(P.bar, P.err, nctas);
  };
  barrier();
  const int rounds = (int)((total + stride - 1) / stride);
  if (CACHE > 0 && rounds <= CACHE) {
    for (int r = 0; r < rounds; r++) {
      const long long gi = first + r * stride;
      if (gi < total) {
        int m;
        const long long cell = cell_of(gi, m);
        const Dev &D = P.d[m];
        const Nb6 n = jacobi_neighbours(D, cell);
        const uint32_t a = (uint32_t)P.arena[m];
        uint32_t *e = s_cache + r * 8 * 256 + t;
        e[0] = a + n.i0; e[256] = a + n.i1; e[512] = a + n.i2;
        e[768] = a + n.i3; e[1024] = a + n.i4; e[1280] = a + n.i5;
        e[1536] = a + (uint32_t)cell;
        const int sc = 1 << s_lev[m];
        const float alpha = (float)(sc * sc) * D.ph.dx * D.ph.dx;
        e[1792] = __float_as_uint(alpha * D.div[cell]);
      }
    }
    for (int it = 0; it < sweeps; it++) {
      const float *src = (it & 1) ? P.pt : P.p;
      float *dst = (it & 1) ? P.p : P.pt;
      for (int r = 0; r < rounds; r++) {
        if (first + r * stride < total) {
          const uint32_t *e = s_cache + r * 8 * 256 + t;
          const Nb6 n = {e[0], e[256], e[512], e[768], e[1024], e[1280]};
          dst[e[1536]] = jacobi_update(src, n, __uint_as_float(e[1792]));
        }
      }
      if (it + 1 < sweeps) barrier();
    }
  } else if constexpr (NB > 0) {
    solve_pipelined<CACHE, NB, CLAIM>(P, s_end, s_lev, s_cache, total, nctas, sweeps, tree);
  } else {
    // staged sweeps, one warp per block: per round each of the CTA's 8 warps
    // takes one block; its 64 cells and 96 face-halo cells go into a 6^3 tile
    // in shared memory, then every cell reads its six neighbours from the
    // tile. The block's description (see fill_block_info) is built once per
    // launch into the dynamic shared memory when it fits, else per sweep.
    // tile strides SX (x), SY (y), 1 (z), interior cell (lx,ly,lz) at
    // (lx+1)*SX + (ly+1)*SY + lz + 2; each lane owns the z-adjacent cell pair
    // c = 2*lane, 2*lane+1, so its own values, divergences and results move
    // as float2 and four of its twelve neighbour reads are float2 tile loads
    constexpr int W = 8, U = DCG_SOLVE_U, SX = DCG_TILE_SX, SY = DCG_TILE_SY, TILE = 5 * SX + 5 * SY + 8;
    __shared__ __align__(16) float s_tile[W][U][TILE];
    __shared__ uint32_t s_scratch[W][U][BI_WORDS];
    const int w = t >> 5, lane = t & 31;
    int oA;
    uint32_t hpk[3], hax[3];
    halo_slots<SX, SY>(lane, oA, hpk, hax);
    const long long nblocks = total >> 6;
    const int rounds_b = (int)((nblocks + (long long)W * nctas - 1) / ((long long)W * nctas));
    // block descriptions: in shared memory when they fit, else built once
    // into the global table P.binfo (indexed by level block) and copied to
    // the warp's scratch when the block comes up
    const bool cached = rounds_b <= CACHE * 2048 / (W * BI_WORDS);
    for (int r = 0; r < rounds_b; r++) {
      const long long gb = ((long long)r * nctas + blockIdx.x) * W + w;
      if (gb >= nblocks) continue;
      if (cached) {
        fill_block_info(P, s_end, s_lev, gb, s_cache + (r * W + w) * BI_WORDS, lane);
      } else {
        fill_block_info(P, s_end, s_lev, gb, s_scratch[w][0], lane);
        __syncwarp();
        if (lane < BI_WORDS) P.binfo[gb * BI_WORDS + lane] = s_scratch[w][0][lane];
        __syncwarp();
      }
    }
    __syncwarp();
    // Passes of U rounds: every lane issues the loads of U blocks before the
    // warp computes any of them; with DCG_SOLVE_PIPE the loads of the next
    // pass are issued before the current pass is computed from its tiles.
    struct Pass {
      float2 own_v[U], dv[U];
      float halo[U][3], alpha[U];
      uint32_t own[U];
      bool act[U];
    };
    const float *src = P.p;
    auto load_pass = [&](int r0, Pass &ps) {
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int r = r0 + u;
        const long long gb = ((long long)r * nctas + blockIdx.x) * W + w;
        ps.act[u] = r < rounds_b && gb < nblocks;  // warp-uniform
        if (!ps.act[u]) continue;
        const uint32_t *bi = cached ? s_cache + (r * W + w) * BI_WORDS : s_scratch[w][u];
        if (!cached) {
          if (lane < BI_WORDS) s_scratch[w][u][lane] = P.binfo[gb * BI_WORDS + lane];
          __syncwarp();
        }
        const uint32_t own = bi[BI_OWN];
        uint32_t addr[3];
        if (bi[BI_CODES] == 0u && (bi[BI_CODES + 1] & 0xFFFFu) == 0u) {
          // all six faces border same-level blocks (warp-uniform fast path)
#pragma unroll
          for (int q = 0; q < 3; q++) addr[q] = bi[BI_FACE + (hax[q] >> 12)] + ((hpk[q] >> 9) & 63);
        } else {
          const uint8_t *codes = reinterpret_cast<const uint8_t *>(bi + BI_CODES);
#pragma unroll
          for (int q = 0; q < 3; q++) {
            const uint32_t pk = hpk[q], ga = hax[q];
            const int f = (int)(ga >> 12);
            const int code = codes[f];
            uint32_t li = code == 0 ? (pk >> 9) & 63 : code == 16 ? (pk >> 15) & 63 : (pk >> 21) & 63;
            if (code > 0 && code < 16) {  // coarser by `code` levels: injection
              const int cx = (int)bi[BI_POS] + (int)(ga & 15) - 1, cy = (int)bi[BI_POS + 1] + (int)((ga >> 4) & 15) - 1,
                        cz = (int)bi[BI_POS + 2] + (int)((ga >> 8) & 15) - 1;
              li = (uint32_t)local_of((cx >> code) & 3, (cy >> code) & 3, (cz >> code) & 3);
            }
            addr[q] = bi[BI_FACE + f] + li;
          }
        }
        ps.own[u] = own;
        ps.alpha[u] = __uint_as_float(bi[BI_ALPHA]);
        ps.own_v[u] = __ldcg(reinterpret_cast<const float2 *>(src + own) + lane);
        ps.halo[u][0] = __ldcg(src + addr[0]);
        ps.halo[u][1] = __ldcg(src + addr[1]);
        ps.halo[u][2] = __ldcg(src + addr[2]);
        ps.dv[u] = reinterpret_cast<const float2 *>(P.div + own)[lane];
      }
    };
    for (int it = 0; it < sweeps; it++) {
      src = (it & 1) ? P.pt : P.p;
      float *dst = (it & 1) ? P.p : P.pt;
      Pass cur, nxt;
      if (DCG_SOLVE_PIPE) load_pass(0, cur);
      for (int r0 = 0; r0 < rounds_b; r0 += U) {
        if (!DCG_SOLVE_PIPE) load_pass(r0, cur);
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!cur.act[u]) continue;
          float *T = s_tile[w][u];
          *reinterpret_cast<float2 *>(T + oA) = cur.own_v[u];
          T[hpk[0] & 511] = cur.halo[u][0];
          T[hpk[1] & 511] = cur.halo[u][1];
          T[hpk[2] & 511] = cur.halo[u][2];
        }
        __syncwarp();
        if (DCG_SOLVE_PIPE) load_pass(r0 + U, nxt);
#pragma unroll
        for (int u = 0; u < U; u++) {
          if (!cur.act[u]) continue;
          const float *T = s_tile[w][u];
          const float2 L = *reinterpret_cast<const float2 *>(T + oA - SX);
          const float2 R = *reinterpret_cast<const float2 *>(T + oA + SX);
          const float2 Dn = *reinterpret_cast<const float2 *>(T + oA - SY);
          const float2 Up = *reinterpret_cast<const float2 *>(T + oA + SY);
          const float Bk = T[oA - 1], Fw = T[oA + 2];
          const float a = cur.own_v[u].x, b = cur.own_v[u].y;
          const float adA = cur.alpha[u] * cur.dv[u].x, adB = cur.alpha[u] * cur.dv[u].y;
          float2 res;
          res.x = div6(L.x + R.x + Dn.x + Up.x + Bk + b - adA);
          res.y = div6(L.y + R.y + Dn.y + Up.y + a + Fw - adB);
          reinterpret_cast<float2 *>(dst + cur.own[u])[lane] = res;
        }
        __syncwarp();
        if (DCG_SOLVE_PIPE) cur = nxt;
      }
      if (it + 1 < sweeps) barrier();
    }
  }
}

// ------------------------------------------------------ staged cell stages
// Divergence (STAGE 2) and pressure application (STAGE 3) one warp per
// block: lanes 0-5 read the block's six face entries of the neighbour table
// once, every lane resolves its three halo cells from them (apron_cell for a
// known face), and the block's values and face halo go through a shared 6^3
// tile, so a cell's six neighbours are tile reads instead of six neighbour
// resolutions. The arithmetic of divergence_cell / apply_pressure_cell is
// kept operation for operation (identical results). Persistent: warps walk
// the allocated blocks of every (member, level) segment.
template <int STAGE>
__global__ void __launch_bounds__(256) k_cells_staged(const __grid_constant__ CellBatch P) {
  constexpr int W = 8, SX = DCG_TILE_SX, SY = DCG_TILE_SY, TILE = 5 * SX + 5 * SY + 8;
  constexpr int NT = STAGE == 2 ? 3 : STAGE == 3 ? 2 : 1;
  __shared__ long long s_end[BMAX * MAXL];
  __shared__ __align__(16) float s_tile[W][NT][TILE];
  // statistics (STAGE 4): per-lane FP64 sums while the warp's member and level
  // stay the same, reduced and added with one atomic per quantity on a change
  double a_res = 0.0, a_mass = 0.0;
  int a_cnt = 0, a_mem = -1, a_lvl = 0;
  auto flush = [&]() {
    double r = a_res, m = a_mass;
    for (int o = 16; o > 0; o >>= 1) {
      r += __shfl_xor_sync(0xffffffffu, r, o);
      m += __shfl_xor_sync(0xffffffffu, m, o);
    }
    const int n = (int)__reduce_add_sync(0xffffffffu, (unsigned)a_cnt);
    stats_flush(P.d[a_mem], r, m, a_lvl, (double)n);
  };  // defect residual (STAGE 6): a_res sums r^2, a_mass div^2 of the warp's member
  auto flush_defect = [&]() {
    double r = a_res, m = a_mass;
    for (int o = 16; o > 0; o >>= 1) {
      r += __shfl_xor_sync(0xffffffffu, r, o);
      m += __shfl_xor_sync(0xffffffffu, m, o);
    }
    if ((threadIdx.x & 31) == 0 && (r != 0.0 || m != 0.0)) {
      double *nrm = P.d[a_mem].dnorm + 2 * P.arg;
      atomicAdd(nrm, r);
      atomicAdd(nrm + 1, m);
    }
  };
  const int nseg = P.n * MAXL;
  for (int i = threadIdx.x; i < nseg; i += blockDim.x) {
    const Dev &D = P.d[i / MAXL];
    const int l = i % MAXL;
    s_end[i] = l < D.g.levels ? __ldcg(D.load + l) : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 1; i < nseg; i++) s_end[i] += s_end[i - 1];
  __syncthreads();
  const long long total = s_end[nseg - 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int oA;
  uint32_t hpk[3], hax[3];
  halo_slots<SX, SY>(lane, oA, hpk, hax);
  const unsigned full = 0xffffffffu;
  // the warp's next block (segment, index, position, face entries, subblock
  // child) is fetched while the current one is computed, so a block waits
  // on one round of loads (its values and face halo) instead of two
  const long long stride = (long long)gridDim.x * W;
  const int fdir = lane == 0 ? 4 : lane == 1 ? 22 : lane == 2 ? 10 : lane == 3 ? 16 : lane == 4 ? 12 : 14;
  int segn = 0;
  uint32_t bn = 0, en = OUT, chn = NONE;
  int4 bpn = make_int4(0, 0, 0, -1);
  auto fetch = [&](long long tt) {
    while (tt >= s_end[segn]) segn++;  // tt grows: the segment only moves forward
    const Dev &Dn = P.d[segn / MAXL];
    bn = (uint32_t)(Dn.g.off[segn % MAXL] + (tt - (segn ? s_end[segn - 1] : 0)));
    bpn = Dn.pos[bn];
    en = lane < 6 ? Dn.nbr[27u * bn + fdir] : OUT;
    chn = Dn.child[8u * bn + (lane >> 2)];
  };
  long long t = (long long)blockIdx.x * W + w;
  if (t < total) fetch(t);
  for (; t < total; t += stride) {
    const int seg = segn;
    const uint32_t b = bn, e = en;
    const int4 bp = bpn;
    const bool leaf = chn == NONE;
    if (t + stride < total) fetch(t + stride);
    const Dev &D = P.d[seg / MAXL];
    const size_t own = (size_t)b * BV;
    size_t hc[3];
#pragma unroll
    for (int q = 0; q < 3; q++) hc[q] = halo_cell(D, b, bp, __shfl_sync(full, e, (int)(hax[q] >> 12)), hpk[q], hax[q]);
    const int scale = 1 << bp.w;
    const float alpha = 0.5f * D.ph.rdx / (float)scale;
    float *T0 = s_tile[w][0], *T1 = s_tile[w][NT > 1 ? 1 : 0];
    if constexpr (STAGE == 6) {
      // the residual of the Jacobi equation (the fixed point of the sweeps:
      // sum6 p - 6 p = alpha div, alpha = (2^L dx)^2 in float as there) for
      // the lane's two cells (every allocated cell): the FP64 sum of the six
      // neighbours in jacobi_neighbours' order (L, R, D, U, B, F) minus 6 p,
      // r = div - lap / alpha, stored in FP32; the FP64 sums of r^2 and
      // div^2 go to the member's norms of correction pass P.arg
      const float2 p2 = reinterpret_cast<const float2 *>(D.p + own)[lane];
      float hp[3];
#pragma unroll
      for (int q = 0; q < 3; q++) hp[q] = D.p[hc[q]];
      *reinterpret_cast<float2 *>(T0 + oA) = p2;
#pragma unroll
      for (int q = 0; q < 3; q++) T0[hpk[q] & 511u] = hp[q];
      __syncwarp();
      if (seg / MAXL != a_mem) {  // warp-uniform
        if (a_mem >= 0) flush_defect();
        a_mem = seg / MAXL;
        a_res = a_mass = 0.0;
      }
      const float2 dv = reinterpret_cast<const float2 *>(D.div + own)[lane];
      const float2 L = *reinterpret_cast<const float2 *>(T0 + oA - SX);
      const float2 R = *reinterpret_cast<const float2 *>(T0 + oA + SX);
      const float2 Dn = *reinterpret_cast<const float2 *>(T0 + oA - SY);
      const float2 U = *reinterpret_cast<const float2 *>(T0 + oA + SY);
      const float Bk = T0[oA - 1], Fw = T0[oA + 2];
      const float al = (float)(scale * scale) * D.ph.dx * D.ph.dx;
      const double lA = (double)L.x + (double)R.x + (double)Dn.x + (double)U.x + (double)Bk + (double)p2.y -
                        6.0 * (double)p2.x;
      const double lB = (double)L.y + (double)R.y + (double)Dn.y + (double)U.y + (double)p2.x + (double)Fw -
                        6.0 * (double)p2.y;
      const double rA = (double)dv.x - lA / (double)al, rB = (double)dv.y - lB / (double)al;
      reinterpret_cast<float2 *>(D.rr + own)[lane] = make_float2((float)rA, (float)rB);
      a_res += rA * rA;
      a_res += rB * rB;
      a_mass += (double)dv.x * (double)dv.x;
      a_mass += (double)dv.y * (double)dv.y;
      __syncwarp();
    } else if constexpr (STAGE == 4) {
      // stats_vals for the lane's two cells: pressure tile, FP32 residual and mass
      const float2 p2 = reinterpret_cast<const float2 *>(D.p + own)[lane];
      float hp[3];
#pragma unroll
      for (int q = 0; q < 3; q++) hp[q] = D.p[hc[q]];
      *reinterpret_cast<float2 *>(T0 + oA) = p2;
#pragma unroll
      for (int q = 0; q < 3; q++) T0[hpk[q] & 511u] = hp[q];
      __syncwarp();
      const unsigned leafmask = __ballot_sync(full, leaf);
      if (leafmask) {  // warp-uniform
        if (seg / MAXL != a_mem || bp.w != a_lvl) {
          if (a_mem >= 0) flush();
          a_mem = seg / MAXL;
          a_lvl = bp.w;
          a_res = a_mass = 0.0;
          a_cnt = 0;
        }
        if (leaf) {
          const float2 dv = reinterpret_cast<const float2 *>(D.div + own)[lane];
          const float2 w2 = reinterpret_cast<const float2 *>(D.w + own)[lane];
          const float qa = q_ld(D, 0, own + 2 * lane), qb = q_ld(D, 0, own + 2 * lane + 1);
          const float2 L = *reinterpret_cast<const float2 *>(T0 + oA - SX);
          const float2 R = *reinterpret_cast<const float2 *>(T0 + oA + SX);
          const float2 Dn = *reinterpret_cast<const float2 *>(T0 + oA - SY);
          const float2 U = *reinterpret_cast<const float2 *>(T0 + oA + SY);
          const float Bk = T0[oA - 1], Fw = T0[oA + 2];
          const float as = D.ph.rdx * D.ph.rdx / (float)(scale * scale);
          const float rA = dv.x - (L.x + R.x + Dn.x + U.x + Bk + p2.y - 6.f * p2.x) * as;
          const float rB = dv.y - (L.y + R.y + Dn.y + U.y + p2.x + Fw - 6.f * p2.y) * as;
          const float s3 = (float)(scale * scale * scale);
          a_res += (double)((float)scale * fabsf(rA));
          a_res += (double)((float)scale * fabsf(rB));
          a_mass += (double)(qa * w2.x * s3);
          a_mass += (double)(qb * w2.y * s3);
          a_cnt += 2;
        }
      }
      __syncwarp();
    } else if constexpr (STAGE == 2) {
      float *T2 = s_tile[w][2];
      const float2 w2 = reinterpret_cast<const float2 *>(D.w + own)[lane];
      const float2 vx = reinterpret_cast<const float2 *>(D.v[0] + own)[lane];
      const float2 vy = reinterpret_cast<const float2 *>(D.v[1] + own)[lane];
      const float2 vz = reinterpret_cast<const float2 *>(D.v[2] + own)[lane];
      float hp[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        float v = D.v[q][hc[q]];
        const uint32_t ga = hax[q];
        const int x = bp.x + (int)(ga & 15u) - 1, y = bp.y + (int)((ga >> 4) & 15u) - 1,
                  z = bp.z + (int)((ga >> 8) & 15u) - 1;
        if (outside(D.g, x, y, z, scale)) v = vel_bc1(D.g, D.ph, v, q, x, y, z, scale);
        hp[q] = D.w[hc[q]] * v;
      }
      *reinterpret_cast<float2 *>(T0 + oA) = make_float2(w2.x * vx.x, w2.y * vx.y);
      *reinterpret_cast<float2 *>(T1 + oA) = make_float2(w2.x * vy.x, w2.y * vy.y);
      const float zA = w2.x * vz.x, zB = w2.y * vz.y;
      *reinterpret_cast<float2 *>(T2 + oA) = make_float2(zA, zB);
      T0[hpk[0] & 511u] = hp[0];
      T1[hpk[1] & 511u] = hp[1];
      T2[hpk[2] & 511u] = hp[2];
      __syncwarp();
      float2 dv = make_float2(0.f, 0.f);
      if (leaf) {
        const float2 L = *reinterpret_cast<const float2 *>(T0 + oA - SX);
        const float2 R = *reinterpret_cast<const float2 *>(T0 + oA + SX);
        const float2 Dn = *reinterpret_cast<const float2 *>(T1 + oA - SY);
        const float2 U = *reinterpret_cast<const float2 *>(T1 + oA + SY);
        const float Bk = T2[oA - 1], Fw = T2[oA + 2];
        dv.x = alpha * (R.x - L.x + U.x - Dn.x + zB - Bk);
        dv.y = alpha * (R.y - L.y + U.y - Dn.y + Fw - zA);
      }
      __syncwarp();
      reinterpret_cast<float2 *>(D.p + own)[lane] = make_float2(0.f, 0.f);
      reinterpret_cast<float2 *>(D.pt + own)[lane] = make_float2(0.f, 0.f);
      reinterpret_cast<float2 *>(D.div + own)[lane] = dv;
    } else {
      const float2 p2 = reinterpret_cast<const float2 *>(D.p + own)[lane];
      const float2 w2 = reinterpret_cast<const float2 *>(D.w + own)[lane];
      float hp[3], hw[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        hp[q] = D.p[hc[q]];
        hw[q] = D.w[hc[q]];
      }
      *reinterpret_cast<float2 *>(T0 + oA) = p2;
      *reinterpret_cast<float2 *>(T1 + oA) = w2;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        T0[hpk[q] & 511u] = hp[q];
        T1[hpk[q] & 511u] = hw[q];
      }
      __syncwarp();
      if (leaf) {
        float2 *V0 = reinterpret_cast<float2 *>(D.v[0] + own) + lane;
        float2 *V1 = reinterpret_cast<float2 *>(D.v[1] + own) + lane;
        float2 *V2 = reinterpret_cast<float2 *>(D.v[2] + own) + lane;
        const float2 v0 = *V0, v1 = *V1, v2 = *V2;
        const float2 PL = *reinterpret_cast<const float2 *>(T0 + oA - SX);
        const float2 PR = *reinterpret_cast<const float2 *>(T0 + oA + SX);
        const float2 PD = *reinterpret_cast<const float2 *>(T0 + oA - SY);
        const float2 PU = *reinterpret_cast<const float2 *>(T0 + oA + SY);
        const float2 WL = *reinterpret_cast<const float2 *>(T1 + oA - SX);
        const float2 WR = *reinterpret_cast<const float2 *>(T1 + oA + SX);
        const float2 WD = *reinterpret_cast<const float2 *>(T1 + oA - SY);
        const float2 WU = *reinterpret_cast<const float2 *>(T1 + oA + SY);
        const float PB = T0[oA - 1], PF = T0[oA + 2], WB = T1[oA - 1], WF = T1[oA + 2];
        float2 o0, o1, o2;
        {
          const float pc = p2.x;
          o0.x = v0.x - alpha * (WR.x * (PR.x - pc) + WL.x * (pc - PL.x));
          o1.x = v1.x - alpha * (WU.x * (PU.x - pc) + WD.x * (pc - PD.x));
          o2.x = v2.x - alpha * (w2.y * (p2.y - pc) + WB * (pc - PB));
        }
        {
          const float pc = p2.y;
          o0.y = v0.y - alpha * (WR.y * (PR.y - pc) + WL.y * (pc - PL.y));
          o1.y = v1.y - alpha * (WU.y * (PU.y - pc) + WD.y * (pc - PD.y));
          o2.y = v2.y - alpha * (WF * (PF - pc) + w2.x * (pc - p2.x));
        }
        *V0 = o0;
        *V1 = o1;
        *V2 = o2;
      }
      __syncwarp();
    }
  }
  if (STAGE == 4 && a_mem >= 0) flush();
  if (STAGE == 6 && a_mem >= 0) flush_defect();
}
// ------------------------------------------------------ staged advection
// Advection one warp per block: the block's 64 cells and its 152 apron cells
// (faces, edges and corners, resolved once per block from the block's 26
// neighbour-table entries as apron_cell does) of the sampled fields go into
// shared 6^3 tiles. A leaf cell whose back-traced sample lies in its own block
// (no finer block there: sample_at then takes the own block) reads its eight
// stencil corners and their fluidities from the tiles; any other leaf cell
// runs the per-cell body (advect_velocity_cell / advect_scalars_cell_t).
// The arithmetic is sample_at's and the per-cell bodies' operation for
// operation, so the results are identical.
// The back-traced point of a cell of the block at bp0 lies in that block
// (sample_at's block offset is 0); sub = the point's subblock. sample_at then
// keeps the block unless that subblock has a child (a descent, level > 0).
__device__ __forceinline__ bool sample_in_own(const Dev &D, int4 bp0, float pxw, float pyw, float pzw, int &sub) {
  const int ix = clampi((int)floorf(pxw), 0, D.g.gx - 1);
  const int iy = clampi((int)floorf(pyw), 0, D.g.gy - 1);
  const int iz = clampi((int)floorf(pzw), 0, D.g.gz - 1);
  const int L0 = bp0.w;
  const int lx = (ix >> L0) - bp0.x, ly = (iy >> L0) - bp0.y, lz = (iz >> L0) - bp0.z;
  sub = (((lx >> 1) & 1) << 2) | (((ly >> 1) & 1) << 1) | ((lz >> 1) & 1);
  return ((((ix >> L0) >> 2) - (bp0.x >> 2)) | (((iy >> L0) >> 2) - (bp0.y >> 2)) |
          (((iz >> L0) >> 2) - (bp0.z >> 2))) == 0;
}
template <int SX, int SY> __device__ __forceinline__ constexpr int tile_delta(int c) {
  return ((c >> 2) & 1) * SX + ((c >> 1) & 1) * SY + (c & 1);
}
// sample_at's weights for a sample in the block at bp (level lev) with the
// corner fluidities read from the tile Wt; off[c] = tile offset of corner c.
struct SmpT {
  int base;  // tile offset of corner 0; corner c at base + tile_delta<SX, SY>(c)
  float wt[8];
  float wAcc;
  int x0, y0, z0, x1, y1, z1, scale;
};
template <int SX, int SY>
__device__ __forceinline__ void sample_tile(int4 bp, int lev, float pxw, float pyw, float pzw, const float *Wt,
                                            SmpT &s) {
  s.scale = 1 << lev;
  const float scaleInv = __int_as_float((127 - lev) << 23);  // 1 / 2^lev, exact
  const float x = pxw * scaleInv - 0.5f, y = pyw * scaleInv - 0.5f, z = pzw * scaleInv - 0.5f;
  const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
  const float dx = x - xf, dy = y - yf, dz = z - zf;
  s.x0 = (int)xf; s.y0 = (int)yf; s.z0 = (int)zf;
  s.x1 = s.x0 + 1; s.y1 = s.y0 + 1; s.z1 = s.z0 + 1;
  const int i = clampi(s.x1 - bp.x, 0, AW - 2);
  const int j = clampi(s.y1 - bp.y, 0, AW - 2);
  const int k = clampi(s.z1 - bp.z, 0, AW - 2);
  s.base = i * SX + j * SY + k + 1;
  const float *Wc = Wt + s.base;
  const float Dx = 1.f - dx, Dy = 1.f - dy, Dz = 1.f - dz;
  s.wt[0] = Wc[tile_delta<SX, SY>(0)] * Dx * Dy * Dz;
  s.wt[1] = Wc[tile_delta<SX, SY>(1)] * Dx * Dy * dz;
  s.wt[2] = Wc[tile_delta<SX, SY>(2)] * Dx * dy * Dz;
  s.wt[3] = Wc[tile_delta<SX, SY>(3)] * Dx * dy * dz;
  s.wt[4] = Wc[tile_delta<SX, SY>(4)] * dx * Dy * Dz;
  s.wt[5] = Wc[tile_delta<SX, SY>(5)] * dx * Dy * dz;
  s.wt[6] = Wc[tile_delta<SX, SY>(6)] * dx * dy * Dz;
  s.wt[7] = Wc[tile_delta<SX, SY>(7)] * dx * dy * dz;
  s.wAcc = s.wt[0] + s.wt[1] + s.wt[2] + s.wt[3] + s.wt[4] + s.wt[5] + s.wt[6] + s.wt[7];
  const float wInv = 1.f / s.wAcc;
#pragma unroll
  for (int c = 0; c < 8; c++) s.wt[c] = s.wt[c] * wInv;
}
__device__ __forceinline__ bool box_inside_t(const Geom &g, const SmpT &s) {
  return s.x0 >= 0 && s.y0 >= 0 && s.z0 >= 0 && s.x1 * s.scale < g.gx && s.y1 * s.scale < g.gy &&
         s.z1 * s.scale < g.gz;
}

// resident CTAs per SM the staged advection's register allocation targets (4:
// 64 registers; measured faster than 3 at 80 registers or 2 at 96)
#ifndef DCG_ADV_MINB
#define DCG_ADV_MINB 4
#endif
// per-cell fallbacks, out of line so that the staged kernel keeps few registers
__device__ __noinline__ void advect_velocity_cell_ool(const Dev &D, long long b, int c) { advect_velocity_cell(D, b, c); }
template <int MODE, int NQ> __device__ __noinline__ void advect_scalars_cell_ool(const Dev &D, long long b, int c) {
  advect_scalars_cell_t<MODE, NQ>(D, b, c);
}

// STAGE 0: velocity (MODE, NQ unused); STAGE 1: scalars of members with
// storage format MODE and NQ scalars (other members have no blocks here).
// Four blocks per CTA pass, 64 threads (two warps) per block, one cell per
// thread; the two warps of a block share its tiles through a named barrier.
// APPLY (STAGE 1 only): the pressure application of the same step first, in
// the same pass: the block's pressure and its face halo go into one more
// tile, each leaf cell computes apply_pressure_cell's velocity from the
// pressure and fluidity tiles, stores it and back-traces with it. The scalar
// advection reads no velocity but its own cell's, so the fused pass gives
// the results of the two stages run one after the other.
template <int STAGE, int MODE, int NQ, bool APPLY = false>
__global__ void __launch_bounds__(256, DCG_ADV_MINB) k_advect_staged(const __grid_constant__ CellBatch P) {
  constexpr int NBK = 4, SX = DCG_TILE_SX, SY = DCG_TILE_SY, TILE = 5 * SX + 5 * SY + 8;
  constexpr int QT = APPLY ? 2 : 1;                  // first scalar tile (tile 1: pressure with APPLY)
  constexpr int NF = STAGE == 0 ? 4 : QT + NQ;  // tile 0: fluidity
  __shared__ long long s_end[BMAX * MAXL];
  __shared__ __align__(16) float s_tile[NBK][NF][TILE];
  __shared__ uint32_t s_slot[2][3][64];  // apron slots a = c + 64 r of thread c (pk ~0u: none)
  const int nseg = P.n * MAXL;
  for (int i = threadIdx.x; i < nseg; i += blockDim.x) {
    const Dev &D = P.d[i / MAXL];
    const int l = i % MAXL;
    const bool mine = STAGE == 0 || (D.g.mixed == MODE && D.g.nq == NQ);
    s_end[i] = (mine && l < D.g.levels) ? __ldcg(D.load + l) : 0;
  }
  if (threadIdx.x < 64) {
    const int c = threadIdx.x;
#pragma unroll 1
    for (int r = 0; r < 3; r++) s_slot[0][r][c] = ~0u, s_slot[1][r][c] = 0u;
    int cnt = 0;
    for (int idx = 0; idx < AW * AW * AW; idx++) {
      const int ax = idx / 36, ay = (idx / 6) % 6, az = idx % 6;
      if (ax > 0 && ax < AW - 1 && ay > 0 && ay < AW - 1 && az > 0 && az < AW - 1) continue;
      if ((cnt & 63) == c) {
        const int same = local_of((ax - 1) & 3, (ay - 1) & 3, (az - 1) & 3);
        const int self = local_of(clampi(ax, 1, BW) - 1, clampi(ay, 1, BW) - 1, clampi(az, 1, BW) - 1);
        const int quirk = local_of(clampi(ax, 1, BW) & 3, clampi(ay, 1, BW) & 3, clampi(az, 1, BW) & 3);
        const int d = dir_of(ax) * 9 + dir_of(ay) * 3 + dir_of(az);
        s_slot[0][cnt >> 6][c] = (uint32_t)(ax * SX + ay * SY + az + 1) | ((uint32_t)same << 9) |
                                 ((uint32_t)self << 15) | ((uint32_t)quirk << 21);
        s_slot[1][cnt >> 6][c] = (uint32_t)ax | ((uint32_t)ay << 4) | ((uint32_t)az << 8) | ((uint32_t)d << 12);
      }
      cnt++;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 1; i < nseg; i++) s_end[i] += s_end[i - 1];
  __syncthreads();
  const long long total = s_end[nseg - 1];
  const int k = threadIdx.x >> 6, c = threadIdx.x & 63, lane = threadIdx.x & 31;
  int oC, lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  oC = (lx + 1) * SX + (ly + 1) * SY + (lz + 1) + 1;
  const unsigned full = 0xffffffffu;
  auto pair_sync = [&]() { asm volatile("bar.sync %0, 64;" ::"r"(1 + k) : "memory"); };
  int seg = 0;
  for (long long t = (long long)blockIdx.x * NBK + k; t < total; t += (long long)gridDim.x * NBK) {
    while (t >= s_end[seg]) seg++;
    const Dev &D = P.d[seg / MAXL];
    const int l = seg % MAXL;
    const uint32_t b = (uint32_t)(D.g.off[l] + (t - (seg ? s_end[seg - 1] : 0)));
    const int4 bp = D.pos[b];
    const size_t own = (size_t)b * BV;
    const size_t cell = own + c;
    const uint32_t e = lane < 27 ? D.nbr[27u * b + lane] : OUT;   // each warp keeps a copy
    const uint32_t ch = lane < 8 ? D.child[8u * b + lane] : NONE;  // the block's subblock children
    float *Wt = s_tile[k][0];
    const float wo = D.w[cell];
    const float va = D.v[0][cell], vb = D.v[1][cell], vc = D.v[2][cell];
    Wt[oC] = wo;
    float qa = 0.f, qb = 0.f;  // own density / temperature (buoyancy)
    if constexpr (STAGE == 0) {
      s_tile[k][1][oC] = va;
      s_tile[k][2][oC] = vb;
      s_tile[k][3][oC] = vc;
      if (D.ph.buoy_a != 0.f || D.ph.buoy_b != 0.f) {
        qa = q_ld(D, 0, cell);
        if (D.g.nq > 1) qb = q_ld(D, 1, cell);
      }
    } else {
      if constexpr (APPLY) s_tile[k][1][oC] = D.p[cell];
#pragma unroll
      for (int kq = 0; kq < NQ; kq++) s_tile[k][QT + kq][oC] = q_ldm<MODE>(D, kq, cell);
    }
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const uint32_t pk = s_slot[0][r][c], ga = s_slot[1][r][c];
      const uint32_t ed = __shfl_sync(full, e, (int)((ga >> 12) & 31u));
      if (pk != ~0u) {
        const size_t ac = halo_cell(D, b, bp, ed, pk, ga);
        const uint32_t at = pk & 511u;
        Wt[at] = D.w[ac];
        if constexpr (STAGE == 0) {
          s_tile[k][1][at] = D.v[0][ac];
          s_tile[k][2][at] = D.v[1][ac];
          s_tile[k][3][at] = D.v[2][ac];
        } else {
          if constexpr (APPLY) {  // pressure on the six faces only
            const uint32_t d = (ga >> 12) & 31u;
            if (d == 4u || d == 22u || d == 10u || d == 16u || d == 12u || d == 14u) s_tile[k][1][at] = D.p[ac];
          }
#pragma unroll
          for (int kq = 0; kq < NQ; kq++) s_tile[k][QT + kq][at] = q_ldm<MODE>(D, kq, ac);
        }
      }
    }
    pair_sync();
    const bool leaf = __shfl_sync(full, ch, c >> 3) == NONE;
    float va2 = va, vb2 = vb, vc2 = vc;  // the velocity the cell back-traces with
    if constexpr (STAGE == 1 && APPLY) {
      if (leaf) {  // apply_pressure_cell's arithmetic, neighbours from the tiles
        const float *Pt = s_tile[k][1];
        const float alpha = 0.5f * D.ph.rdx / (float)(1 << bp.w);
        const float pc = Pt[oC];
        va2 = va - alpha * (Wt[oC + SX] * (Pt[oC + SX] - pc) + Wt[oC - SX] * (pc - Pt[oC - SX]));
        vb2 = vb - alpha * (Wt[oC + SY] * (Pt[oC + SY] - pc) + Wt[oC - SY] * (pc - Pt[oC - SY]));
        vc2 = vc - alpha * (Wt[oC + 1] * (Pt[oC + 1] - pc) + Wt[oC - 1] * (pc - Pt[oC - 1]));
        D.v[0][cell] = va2;
        D.v[1][cell] = vb2;
        D.v[2][cell] = vc2;
      }
    }
    float px = 0.f, py = 0.f, pz = 0.f;
    bool fast = false;
    int sub = 0;
    if (leaf) {
      const float scale = (float)(1 << bp.w);
      const float alpha = D.ph.dt * D.ph.rdx;
      px = ((float)(bp.x + lx) + 0.5f) * scale - va2 * alpha;
      py = ((float)(bp.y + ly) + 0.5f) * scale - vb2 * alpha;
      pz = ((float)(bp.z + lz) + 0.5f) * scale - vc2 * alpha;
      fast = sample_in_own(D, bp, px, py, pz, sub);
    }
    // the sample's subblock must have no child (else sample_at descends)
    const bool sub_leaf = __shfl_sync(full, ch, sub) == NONE;
    fast = fast && (bp.w == 0 || sub_leaf);
    if constexpr (STAGE == 0) {
      if (leaf && !fast) {
        advect_velocity_cell_ool(D, b, c);
      } else {
        float o0 = 0.f, o1 = 0.f, o2 = 0.f;
        if (leaf) {
          SmpT s;
          sample_tile<SX, SY>(bp, bp.w, px, py, pz, Wt, s);
          if (!(s.wAcc < 1e-6f)) {
            const bool inside = box_inside_t(D.g, s);
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
              const int o = s.base + tile_delta<SX, SY>(kk);
              float vx = s_tile[k][1][o], vy = s_tile[k][2][o], vz = s_tile[k][3][o];
              if (!inside) {
                const int x = (kk & 4) ? s.x1 : s.x0, y = (kk & 2) ? s.y1 : s.y0, z = (kk & 1) ? s.z1 : s.z0;
                vel_bc(D.g, D.ph, vx, vy, vz, x, y, z, s.scale);
              }
              if (kk == 0) {
                o0 = vx * s.wt[0]; o1 = vy * s.wt[0]; o2 = vz * s.wt[0];
              } else {
                o0 = o0 + vx * s.wt[kk]; o1 = o1 + vy * s.wt[kk]; o2 = o2 + vz * s.wt[kk];
              }
            }
          }
          if (D.ph.buoy_a != 0.f || D.ph.buoy_b != 0.f) {
            float f = -D.ph.buoy_a * qa;
            if (D.g.nq > 1) f = f + D.ph.buoy_b * (qb - D.ph.t_amb);
            o1 = o1 + D.ph.dt * f;
          }
        }
        D.tv[0][cell] = o0;
        D.tv[1][cell] = o1;
        D.tv[2][cell] = o2;
      }
    } else {
      if (leaf && !fast) {
        advect_scalars_cell_ool<MODE, NQ>(D, b, c);
      } else {
        float o[NQ];
#pragma unroll
        for (int kq = 0; kq < NQ; kq++) o[kq] = 0.f;
        if (leaf) {
          SmpT s;
          sample_tile<SX, SY>(bp, bp.w, px, py, pz, Wt, s);
          if (!(s.wAcc < 1e-6f)) {
            const bool inside = box_inside_t(D.g, s);
#pragma unroll
            for (int kk = 0; kk < 8; kk++) {
              const int x = (kk & 4) ? s.x1 : s.x0, y = (kk & 2) ? s.y1 : s.y0, z = (kk & 1) ? s.z1 : s.z0;
              const int mode = inside ? 0 : q_bc_mode(D.g, D.ph, x, y, z, s.scale);
#pragma unroll
              for (int kq = 0; kq < NQ; kq++) {
                const float qc = mode == 0 ? s_tile[k][QT + kq][s.base + tile_delta<SX, SY>(kk)]
                                           : (mode == 1 && kq == 0 ? D.ph.d_emit : 0.f);
                o[kq] = (kk == 0) ? qc * s.wt[0] : o[kq] + qc * s.wt[kk];
              }
            }
          }
          if (D.ph.em_n > 0)
            o[0] = o[0] + D.ph.dt * emission_at(D.g, D.ph, bp.x + lx, bp.y + ly, bp.z + lz, 1 << bp.w);
          if (D.ph.src) {
            if (in_source(D.ph, bp.x + lx, bp.y + ly, bp.z + lz, 1 << bp.w))
#pragma unroll
              for (int kq = 0; kq < NQ; kq++) o[kq] = src_value_at(D.ph, kq, bp.x + lx, bp.y + ly, bp.z + lz, bp.w);
          }
        }
#pragma unroll
        for (int kq = 0; kq < NQ; kq++) tq_stm<MODE>(D, kq, cell, o[kq]);
      }
    }
    pair_sync();  // the tiles are refilled for the next block
  }
}
template <int STAGE, int MODE, int NQ, bool APPLY = false> static unsigned advect_grid() {
  static unsigned g = 0;
  if (!g) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_advect_staged<STAGE, MODE, NQ, APPLY>, 256, 0);
    g = (unsigned)(sms * (occ > 0 ? occ : 1));
  }
  return g;
}
// the scalar advection, one launch per storage format and scalar count present
template <bool APPLY> static void launch_advect_scalars_staged(const CellBatch &P, cudaStream_t st) {
  bool has[3][2] = {};
  for (int i = 0; i < P.n; i++) has[P.d[i].g.mixed][P.d[i].g.nq == 3 ? 1 : 0] = true;
  if (has[0][0]) k_advect_staged<1, 0, 1, APPLY><<<advect_grid<1, 0, 1, APPLY>(), 256, 0, st>>>(P);
  if (has[0][1]) k_advect_staged<1, 0, 3, APPLY><<<advect_grid<1, 0, 3, APPLY>(), 256, 0, st>>>(P);
  if (has[1][0]) k_advect_staged<1, 1, 1, APPLY><<<advect_grid<1, 1, 1, APPLY>(), 256, 0, st>>>(P);
  if (has[1][1]) k_advect_staged<1, 1, 3, APPLY><<<advect_grid<1, 1, 3, APPLY>(), 256, 0, st>>>(P);
  if (has[2][0]) k_advect_staged<1, 2, 1, APPLY><<<advect_grid<1, 2, 1, APPLY>(), 256, 0, st>>>(P);
  if (has[2][1]) k_advect_staged<1, 2, 3, APPLY><<<advect_grid<1, 2, 3, APPLY>(), 256, 0, st>>>(P);
}
static void launch_advect_staged(int stage, const CellBatch &P, cudaStream_t st) {
  if (stage == 0) k_advect_staged<0, 0, 1><<<advect_grid<0, 0, 1>(), 256, 0, st>>>(P);
  else if (stage == 5) launch_advect_scalars_staged<true>(P, st);
  else launch_advect_scalars_staged<false>(P, st);
}

static unsigned staged_grid(int stage) {
  static unsigned g[4] = {0, 0, 0, 0};
  const int i = stage == 2 ? 0 : stage == 3 ? 1 : stage == 4 ? 2 : 3;
  if (!g[i]) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (stage == 2) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cells_staged<2>, 256, 0);
    else if (stage == 3) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cells_staged<3>, 256, 0);
    else if (stage == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cells_staged<4>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cells_staged<6>, 256, 0);
    g[i] = (unsigned)(sms * (occ > 0 ? occ : 1));
  }
  return g[i];
}

// Self-check of div6 and its packed form div6x2: every binary32 bit pattern
// against the IEEE division
// (NaN results compare equal whatever their payload).
__global__ void __launch_bounds__(256) k_check_div6(unsigned long long *bad) {
  unsigned long long n = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long u = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; u < (1ull << 32);
       u += stride) {
    const float x = __uint_as_float((uint32_t)u);
    const float a = x / 6.f, b = div6(x);
    // the packed form, with x in either component (the other a different input)
    const float2 p = div6x2(make_float2(x, __uint_as_float((uint32_t)u ^ 0x80000001u)));
    const float2 p2 = div6x2(make_float2(__uint_as_float((uint32_t)u + 0x01234567u), x));
    const bool ok = (__float_as_uint(a) == __float_as_uint(b) || (a != a && b != b)) &&
                    (__float_as_uint(a) == __float_as_uint(p.x) || (a != a && p.x != p.x)) &&
                    (__float_as_uint(a) == __float_as_uint(p2.y) || (a != a && p2.y != p2.y));
    if (!ok) {
      n++;
      atomicMin(bad + 1, u);
    }
  }
  if (n) atomicAdd(bad, n);
}
void launch_check_div6(unsigned long long *bad, int sms, cudaStream_t st) {
  k_check_div6<<<(unsigned)(sms > 0 ? sms * 8 : 1024), 256, 0, st>>>(bad);
}

// Self-check of the bounded grid-barrier wait: CTA `absent` leaves without
// arriving, so the others wait on a generation word that nothing advances,
// give up after `limit` polls and record DCG_DEVERR_TIMEOUT; the second
// barrier must then return at once (the error bit short-cuts it).
__global__ void __launch_bounds__(64) k_barrier_probe(uint32_t *bar, uint32_t *errw, unsigned limit,
                                                      unsigned absent) {
  if (blockIdx.x == absent) return;
  grid_barrier(bar, errw, gridDim.x, limit);
  grid_barrier(bar, errw, gridDim.x, limit);
}
int launch_barrier_probe(uint32_t *bar, uint32_t *errw, unsigned limit, unsigned nctas, cudaStream_t st) {
  unsigned absent = nctas - 1;
  void *args[] = {&bar, &errw, &limit, &absent};
  return (int)cudaLaunchCooperativeKernel((const void *)k_barrier_probe, dim3(nctas), dim3(64), args, 0, st);
}

template <int TB, int STAGE> static unsigned persist_grid() {
  static unsigned g = 0;
  if (!g) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_cells_persist<TB, STAGE>, 64 * TB, 0);
    g = (unsigned)(sms * (occ > 0 ? occ : 1));
  }
  return g;
}
template <int TB>
static void cells_persist_tb(int stage, const CellBatch &P, cudaStream_t st) {
  switch (stage) {
    case 0: k_cells_persist<TB, 0><<<persist_grid<TB, 0>(), 64 * TB, 0, st>>>(P); break;
    case 1: k_cells_persist<TB, 1><<<persist_grid<TB, 1>(), 64 * TB, 0, st>>>(P); break;
    case 2: k_cells_persist<TB, 2><<<persist_grid<TB, 2>(), 64 * TB, 0, st>>>(P); break;
    case 3: k_cells_persist<TB, 3><<<persist_grid<TB, 3>(), 64 * TB, 0, st>>>(P); break;
    default: k_cells_persist<TB, 4><<<persist_grid<TB, 4>(), 64 * TB, 0, st>>>(P); break;
  }
}
template <int TB>
static void cells_batch_tb(int stage, const CellBatch &P, unsigned grid, cudaStream_t st) {
  switch (stage) {
    case 0: k_cells_batch<TB, 0><<<grid, 64 * TB, 0, st>>>(P); break;
    case 1: k_cells_batch<TB, 1><<<grid, 64 * TB, 0, st>>>(P); break;
    case 2: k_cells_batch<TB, 2><<<grid, 64 * TB, 0, st>>>(P); break;
    case 3: k_cells_batch<TB, 3><<<grid, 64 * TB, 0, st>>>(P); break;
    default: k_cells_batch<TB, 4><<<grid, 64 * TB, 0, st>>>(P); break;
  }
}
void launch_cells_batch(int stage, CellBatch &P, int tile, cudaStream_t st, bool persistent) {
  if (tile == 1 || stage >= 5) {  // staged, one warp per block (5, 6: staged only)
    if (stage < 2 || stage == 5) launch_advect_staged(stage, P, st);
    else if (stage == 2) k_cells_staged<2><<<staged_grid(2), 256, 0, st>>>(P);
    else if (stage == 3) k_cells_staged<3><<<staged_grid(3), 256, 0, st>>>(P);
    else if (stage == 4) k_cells_staged<4><<<staged_grid(4), 256, 0, st>>>(P);
    else k_cells_staged<6><<<staged_grid(6), 256, 0, st>>>(P);
    return;
  }
  if (tile != 2 && tile != 8) tile = 4;
  if (persistent) {
    if (tile == 2) cells_persist_tb<2>(stage, P, st);
    else if (tile == 8) cells_persist_tb<8>(stage, P, st);
    else cells_persist_tb<4>(stage, P, st);
    return;
  }
  long long acc = 0;
  for (int m = 0; m < P.n; m++) {
    acc += (P.d[m].g.B + tile - 1) / tile;
    P.end[m] = acc;
  }
  if (acc == 0) return;
  if (tile == 2) cells_batch_tb<2>(stage, P, (unsigned)acc, st);
  else if (tile == 8) cells_batch_tb<8>(stage, P, (unsigned)acc, st);
  else cells_batch_tb<4>(stage, P, (unsigned)acc, st);
}
void launch_restrict_batch(RestrictBatch &P, cudaStream_t st) {
  long long acc = 0;
  for (int m = 0; m < P.n; m++) {
    if (P.level < P.d[m].g.levels - 1) acc += (8 * P.d[m].g.budget[P.level] + 255) / 256;
    P.end[m] = acc;
  }
  if (acc > 0) k_restrict_batch<<<(unsigned)acc, 256, 0, st>>>(P);
}

template <int C, int NB, int MB = DCG_PIPE_MINB, int CLAIM = DCG_PIPE_CLAIM>
static int solve_batch_occupancy() {
  // static + dynamic shared memory above 48 KB needs the opt-in
  const int smem = C * 8 * 256 * 4;
  if (smem > 0 && cudaFuncSetAttribute(k_level_solve_batch<C, NB, MB, CLAIM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return 0;
  int a = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_level_solve_batch<C, NB, MB, CLAIM>, 256, smem) != cudaSuccess)
    return 0;
  return a;
}
// solve variants: cache depth 0, 3, 4 or 8 (cells per thread of the small-level
// path; 8 KB of dynamic shared memory each); 16 + c: pipelined staged sweeps
// with two tile buffers per warp (registers for 3 CTAs per SM, two blocks per
// claim), 32 + c: three buffers, 64 + c: two buffers with registers for 5
// CTAs per SM, 80 + c: two buffers, registers for 4 CTAs per SM, one block per
// claim
static int solve_occupancy(int cache) {
  switch (cache) {
    case 8: return solve_batch_occupancy<8, 0>();
    case 4: return solve_batch_occupancy<4, 0>();
    case 3: return solve_batch_occupancy<3, 0>();
    case 0: return solve_batch_occupancy<0, 0>();
    case 16: return solve_batch_occupancy<0, 2>();
    case 32: return solve_batch_occupancy<0, 3>();
    case 16 + 2: return solve_batch_occupancy<2, 2>();
    case 16 + 3: return solve_batch_occupancy<3, 2>();
    case 32 + 2: return solve_batch_occupancy<2, 3>();
    case 32 + 3: return solve_batch_occupancy<3, 3>();
    case 64: return solve_batch_occupancy<0, 2, 5>();
    case 64 + 2: return solve_batch_occupancy<2, 2, 5>();
    case 80 + 3: return solve_batch_occupancy<3, 2, 4, 1>();
    default: return 0;
  }
}
bool solve_variant_valid(int cache) {
  return cache == 0 || cache == 3 || cache == 4 || cache == 8 || cache == 16 || cache == 18 || cache == 19 ||
         cache == 32 || cache == 34 || cache == 35 || cache == 64 || cache == 66 || cache == 83;
}
int batch_solve_grid(int sms, int cache, int ctas_per_sm) {
  const int occ = solve_occupancy(cache);
  if (occ <= 0) return 0;
  if (ctas_per_sm < 0) return std::max(1, sms / -ctas_per_sm);  // one CTA per -ctas_per_sm SMs
  const int k = (ctas_per_sm > 0 && ctas_per_sm < occ) ? ctas_per_sm : occ;
  return k * sms;
}
void launch_level_solve_batch(const SolveBatch &P, int round, int sweeps, int grid, int cache, int tree,
                              cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(256);
  if (!solve_variant_valid(cache)) cache = 0;
  cfg.dynamicSmemBytes = (size_t)(cache & 15) * 8 * 256 * 4;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  switch (cache) {
    case 8: cudaLaunchKernelEx(&cfg, k_level_solve_batch<8, 0>, P, round, sweeps, tree); break;
    case 4: cudaLaunchKernelEx(&cfg, k_level_solve_batch<4, 0>, P, round, sweeps, tree); break;
    case 3: cudaLaunchKernelEx(&cfg, k_level_solve_batch<3, 0>, P, round, sweeps, tree); break;
    case 16: cudaLaunchKernelEx(&cfg, k_level_solve_batch<0, 2>, P, round, sweeps, tree); break;
    case 32: cudaLaunchKernelEx(&cfg, k_level_solve_batch<0, 3>, P, round, sweeps, tree); break;
    case 18: cudaLaunchKernelEx(&cfg, k_level_solve_batch<2, 2>, P, round, sweeps, tree); break;
    case 19: cudaLaunchKernelEx(&cfg, k_level_solve_batch<3, 2>, P, round, sweeps, tree); break;
    case 34: cudaLaunchKernelEx(&cfg, k_level_solve_batch<2, 3>, P, round, sweeps, tree); break;
    case 35: cudaLaunchKernelEx(&cfg, k_level_solve_batch<3, 3>, P, round, sweeps, tree); break;
    case 64: cudaLaunchKernelEx(&cfg, k_level_solve_batch<0, 2, 5>, P, round, sweeps, tree); break;
    case 66: cudaLaunchKernelEx(&cfg, k_level_solve_batch<2, 2, 5>, P, round, sweeps, tree); break;
    case 83: cudaLaunchKernelEx(&cfg, k_level_solve_batch<3, 2, 4, 1>, P, round, sweeps, tree); break;
    default: cudaLaunchKernelEx(&cfg, k_level_solve_batch<0, 0>, P, round, sweeps, tree); break;
  }
}

}  // namespace dcg
