// k_adjoint.cu — adjoint (transpose) of the density path of one step.
//
// With the flow and the grid topology of a step held fixed (topology as
// recorded, not differentiated), the step maps the density linearly:
//   q_t = R_t ( A_t ( Prop_t (q_{t-1}) ) + dt * S_t E ),
// Prop_t = values of the blocks the adaptation moved or created, interpolated
//          from their parents (k_propagate),
// A_t    = semi-Lagrangian advection with the step's projected velocity
//          (trilinear, fluidity-weighted, renormalised; boundary cells that
//          pass the scalar through), source cells overwritten,
// S_t    = trilinear splat of the emission map E into the bottom band,
// R_t    = fine-to-coarse restriction (8-cell means).
// The kernels below apply R_t^T, A_t^T / S_t^T (scatters with atomics) and
// Prop_t^T in the reverse order, using the state after the step (its
// velocity, fluidity, topology and touched-block list), plus the transpose of
// the dense resampling used by losses on the dense grid.
#include "dcg_dev.cuh"
#include "dcg_kernels.h"

namespace dcg {

// restriction transpose for one level: one thread per child subblock
__global__ void __launch_bounds__(256) k_adj_restrict(Dev D, int level, float *lam) {
  const long long sl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (sl >= 8 * D.g.budget[level]) return;
  const long long b = D.g.off[level] + (sl >> 3);
  if (D.pos[b].w != level) return;
  const uint32_t par = D.parent[b];
  if (par == NONE) return;
  const int s = (int)(sl & 7);
  const size_t pc = (size_t)par * 8 + s;
  const size_t base = (size_t)b * BV + 8 * s;
  const float lp = lam[pc] * 0.125f;
#pragma unroll
  for (int i = 0; i < 8; i++) lam[base + i] += lp;
  lam[pc] = 0.f;
}

// q_bc passes the sampled scalar through (identity) at this corner
__device__ inline bool q_passes(const Geom &g, const Phys &P, int x, int y, int z, int scale) {
  if (in_inlet(g, P, x, y, z, scale)) return false;
  if (P.wind && yz_inside(g, y, z, scale)) {
    if (x < 0) return false;
    if (x * scale >= g.gx) return true;
  }
  return !outside(g, x, y, z, scale);
}

// transpose of emission_at: adds g * d(emission)/d(E[i]) to lam_em[i]
__device__ inline void emission_adjoint(const Geom &g, const Phys &P, int x, int y, int z, int scale, float gval,
                                        float *lam_em) {
  const float s = (float)scale;
  const float yw = ((float)y + 0.5f) * s;
  if (!(yw < P.em_band)) return;
  const float xw = ((float)x + 0.5f) * s, zw = ((float)z + 0.5f) * s;
  const int n = P.em_n;
  const float top = (float)(n - 1);
  const float u = clampf_(xw * ((float)n / (float)g.gx) - 0.5f, 0.f, top);
  const float v = clampf_(yw * ((float)n / P.em_band) - 0.5f, 0.f, top);
  const float w = clampf_(zw * ((float)n / (float)g.gz) - 0.5f, 0.f, top);
  const int i0 = (int)floorf(u), j0 = (int)floorf(v), k0 = (int)floorf(w);
  const int i1 = i0 + 1 < n ? i0 + 1 : n - 1, j1 = j0 + 1 < n ? j0 + 1 : n - 1, k1 = k0 + 1 < n ? k0 + 1 : n - 1;
  const float fu = u - (float)i0, fv = v - (float)j0, fw = w - (float)k0;
  const int I[2] = {i0, i1}, J[2] = {j0, j1}, K[2] = {k0, k1};
  const float WU[2] = {1.f - fu, fu}, WV[2] = {1.f - fv, fv}, WW[2] = {1.f - fw, fw};
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int a = (c >> 2) & 1, bb = (c >> 1) & 1, cc = c & 1;
    atomicAdd(lam_em + ((size_t)K[cc] * n + J[bb]) * n + I[a], gval * WU[a] * WV[bb] * WW[cc]);
  }
}

// advection + emission transpose: leaf cell c scatters lam_in[c] to the cells
// its back-traced sample read, and dt * lam_in[c] to the emission map
__global__ void __launch_bounds__(256) k_adj_advect_density(Dev D, const float *lam_in, float *lam_out, float *lam_em) {
  const long long b = (long long)blockIdx.x * 4 + (threadIdx.x >> 6);
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  const float l = lam_in[cell];
  if (l == 0.f) return;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz, scale = 1 << bp.w;
  if (D.ph.src && in_source(D.ph, x, y, z, scale)) return;
  if (D.ph.em_n > 0 && lam_em) emission_adjoint(D.g, D.ph, x, y, z, scale, D.ph.dt * l, lam_em);
  float px, py, pz;
  back_trace(D, bp, c, cell, px, py, pz);
  Smp s;
  sample_at(D, (uint32_t)b, bp, px, py, pz, s);
  if (s.wAcc < 1e-6f) return;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int cx = (k & 4) ? s.x1 : s.x0, cy = (k & 2) ? s.y1 : s.y0, cz = (k & 1) ? s.z1 : s.z0;
    if (q_passes(D.g, D.ph, cx, cy, cz, s.scale)) atomicAdd(lam_out + s.idx[k], l * s.wt[k]);
  }
}

// propagation transpose for the touched blocks of one level
__global__ void __launch_bounds__(256) k_adj_propagate(Dev D, int level, float *lam) {
  const long long nt = D.ctr[C_TOUCHED];
  const int c = threadIdx.x & 63;
  for (long long t = (long long)blockIdx.x * 4 + (threadIdx.x >> 6); t < nt; t += (long long)gridDim.x * 4) {
    const uint32_t b = D.touched[t];
    if (b == NONE) continue;
    const int4 bp = D.pos[b];
    if (bp.w != level) continue;
    const uint32_t par = D.parent[b];
    if (par == NONE) continue;
    const uint32_t pb = par >> 3;
    const int4 pbp = D.pos[pb];
    int lx, ly, lz;
    local_xyz(c, lx, ly, lz);
    const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz;
    const int ax = 1 + (x / 2) % BW, ay = 1 + (y / 2) % BW, az = 1 + (z / 2) % BW;
    const int i = x % 2 ? 1 : -1, j = y % 2 ? 1 : -1, k = z % 2 ? 1 : -1;
    const size_t cell = (size_t)b * BV + c;
    const float l = lam[cell];
    lam[cell] = 0.f;
    if (l == 0.f) continue;
    atomicAdd(lam + apron_cell(D, pb, pbp, ax, ay, az), (27.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax, ay, az + k), (9.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax, ay + j, az), (9.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax + i, ay, az), (9.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax, ay + j, az + k), (3.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax + i, ay, az + k), (3.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax + i, ay + j, az), (3.f / 64.f) * l);
    atomicAdd(lam + apron_cell(D, pb, pbp, ax + i, ay + j, az + k), (1.f / 64.f) * l);
  }
}

// dense resampling transpose: every finest cell adds its adjoint to the leaf
// cell that covers it
__global__ void __launch_bounds__(256) k_adj_dense(Dev D, const float *lam_dense, float *lam) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)D.g.gx * D.g.gy * D.g.gz;
  if (i >= n) return;
  const float l = lam_dense[i];
  if (l == 0.f) return;
  const int x = (int)(i % D.g.gx), y = (int)((i / D.g.gx) % D.g.gy), z = (int)(i / ((long long)D.g.gx * D.g.gy));
  int lev;
  const uint32_t b = locate(D, x, y, z, 0, lev);
  const int4 bp = D.pos[b];
  atomicAdd(lam + (size_t)b * BV + local_of((x >> lev) - bp.x, (y >> lev) - bp.y, (z >> lev) - bp.z), l);
}

void launch_adjoint_step(const Dev &D, float *lam_in_scratch, float *lam_out, float *lam_em, int sms,
                         cudaStream_t st) {
  for (int level = D.g.levels - 2; level >= 0; level--) {
    const long long n = 8 * D.g.budget[level];
    k_adj_restrict<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(D, level, lam_in_scratch);
  }
  cudaMemsetAsync(lam_out, 0, (size_t)D.g.B * BV * sizeof(float), st);
  k_adj_advect_density<<<(unsigned)((D.g.B + 3) / 4), 256, 0, st>>>(D, lam_in_scratch, lam_out, lam_em);
  const unsigned gs = (unsigned)(sms > 0 ? sms * 4 : 512);
  for (int level = 0; level <= D.g.levels - 2; level++) k_adj_propagate<<<gs, 256, 0, st>>>(D, level, lam_out);
}
void launch_adjoint_dense(const Dev &D, const float *lam_dense, float *lam, cudaStream_t st) {
  const long long n = (long long)D.g.gx * D.g.gy * D.g.gz;
  k_adj_dense<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(D, lam_dense, lam);
}

}  // namespace dcg
