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

// ===========================================================================
// Full adjoint of one step: velocity advection (field and back-traced
// positions), buoyancy, propagation, divergence, the cascade (each Jacobi
// sweep and prolongation transposed, in reverse order), the pressure
// gradient, and the scalar advection (field and positions), with the
// topology of the step recorded. The step is nonlinear in the velocity (the
// back-traced positions move the trilinear weights); the transposes apply its
// Jacobian at the recorded state. The weights' derivative with respect to
// the sample position is taken inside the sampled cell (the trilinear weights
// are piecewise linear; the located block and the cell are held fixed).
namespace dcg {

// derivative data of a sample's weights: dW[a][c] = d(w_c * trilinear_c) /
// d(fractional coordinate a); G[a] = sum_c dW[a][c]. The normalised weight's
// derivative is (dW[a][c] - wt[c] * G[a]) / wAcc.
struct SmpD {
  float dW[3][8];
  float G[3];
};
__device__ inline void sample_derivs(const Dev &D, const Smp &s, float pxw, float pyw, float pzw, SmpD &d) {
  const float scaleInv = 1.f / (float)s.scale;
  const float x = pxw * scaleInv - 0.5f, y = pyw * scaleInv - 0.5f, z = pzw * scaleInv - 0.5f;
  const float dx = x - floorf(x), dy = y - floorf(y), dz = z - floorf(z);
  const float Dx = 1.f - dx, Dy = 1.f - dy, Dz = 1.f - dz;
  d.G[0] = d.G[1] = d.G[2] = 0.f;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const float wc = D.w[s.idx[c]];
    const float X = (c & 4) ? dx : Dx, Y = (c & 2) ? dy : Dy, Z = (c & 1) ? dz : Dz;
    const float sx = (c & 4) ? 1.f : -1.f, sy = (c & 2) ? 1.f : -1.f, sz = (c & 1) ? 1.f : -1.f;
    d.dW[0][c] = wc * sx * Y * Z;
    d.dW[1][c] = wc * X * sy * Z;
    d.dW[2][c] = wc * X * Y * sz;
    d.G[0] += d.dW[0][c];
    d.G[1] += d.dW[1][c];
    d.G[2] += d.dW[2][c];
  }
}

__device__ __forceinline__ long long adj_block() { return (long long)blockIdx.x * 4 + (threadIdx.x >> 6); }

// Scalar advection transpose (state after the adaptation, velocity after the
// projection, D.q = the scalars the advection read): leaf cell c scatters the
// adjoint of each advected scalar to the cells its sample read (lamq0, nq
// planes of nc), dt * adjoint of the density to the emission map, and adds
// the derivative through its back-traced position to the adjoint of its own
// velocity (lamv, 3 planes). Source cells are overwritten by the step: no
// dependence.
__global__ void __launch_bounds__(256) k_adj_scalars_full(Dev D, const float *lamq, float *lamq0, float *lamv,
                                                          float *lam_em, size_t nc) {
  const long long b = adj_block();
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  float lq[3];
  bool any = false;
  for (int k = 0; k < D.g.nq; k++) {
    lq[k] = lamq[k * nc + cell];
    any |= lq[k] != 0.f;
  }
  if (!any) return;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int scale0 = 1 << bp.w;
  if (D.ph.src && in_source(D.ph, bp.x + lx, bp.y + ly, bp.z + lz, scale0)) return;
  if (D.ph.em_n > 0 && lam_em && lq[0] != 0.f)
    emission_adjoint(D.g, D.ph, bp.x + lx, bp.y + ly, bp.z + lz, scale0, D.ph.dt * lq[0], lam_em);
  float px, py, pz;
  back_trace(D, bp, c, cell, px, py, pz);
  Smp s;
  sample_at(D, (uint32_t)b, bp, px, py, pz, s);
  if (s.wAcc < 1e-6f) return;
  SmpD d;
  sample_derivs(D, s, px, py, pz, d);
  float gsum[3] = {0.f, 0.f, 0.f};
  for (int k = 0; k < D.g.nq; k++) {
    if (lq[k] == 0.f) continue;
    float out = 0.f, H[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int cc = 0; cc < 8; cc++) {
      int x, y, z;
      corner_of(s, cc, x, y, z);
      const float raw = D.q[k][s.idx[cc]];
      const float val = q_bc(D.g, D.ph, raw, k, x, y, z, s.scale);
      out += s.wt[cc] * val;
      H[0] += d.dW[0][cc] * val;
      H[1] += d.dW[1][cc] * val;
      H[2] += d.dW[2][cc] * val;
      if (q_passes(D.g, D.ph, x, y, z, s.scale)) atomicAdd(lamq0 + k * nc + s.idx[cc], lq[k] * s.wt[cc]);
    }
#pragma unroll
    for (int a = 0; a < 3; a++) gsum[a] += lq[k] * (H[a] - out * d.G[a]) / s.wAcc;
  }
  const float f = -(D.ph.dt * D.ph.rdx) / (float)s.scale;
#pragma unroll
  for (int a = 0; a < 3; a++) lamv[a * nc + cell] += f * gsum[a];
}

// Velocity advection + buoyancy transpose (the state before the step:
// topology, velocity, scalars and fluidity of its start): leaf cell c
// scatters the adjoint of its advected velocity (lamtv, 3 planes) to the
// cells its sample read and, through its back-traced position, to its own
// velocity (lamv0, 3 planes, atomics: other cells scatter there too); the
// buoyancy term adds -dt alpha and dt beta times the adjoint of v.y to the
// density and temperature of the cell (lamq0).
__global__ void __launch_bounds__(256) k_adj_velocity_full(Dev D, const float *lamtv, float *lamv0, float *lamq0,
                                                           size_t nc) {
  const long long b = adj_block();
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  const float l[3] = {lamtv[cell], lamtv[nc + cell], lamtv[2 * nc + cell]};
  if (l[0] == 0.f && l[1] == 0.f && l[2] == 0.f) return;
  if (D.ph.buoy_a != 0.f || D.ph.buoy_b != 0.f) {
    lamq0[cell] += -D.ph.dt * D.ph.buoy_a * l[1];
    if (D.g.nq > 1) lamq0[nc + cell] += D.ph.dt * D.ph.buoy_b * l[1];
  }
  float px, py, pz;
  back_trace(D, bp, c, cell, px, py, pz);
  Smp s;
  sample_at(D, (uint32_t)b, bp, px, py, pz, s);
  if (s.wAcc < 1e-6f) return;
  SmpD d;
  sample_derivs(D, s, px, py, pz, d);
  float gsum[3] = {0.f, 0.f, 0.f};
  for (int comp = 0; comp < 3; comp++) {
    if (l[comp] == 0.f) continue;
    float out = 0.f, H[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int cc = 0; cc < 8; cc++) {
      int x, y, z;
      corner_of(s, cc, x, y, z);
      const float val = vel_bc1(D.g, D.ph, D.v[comp][s.idx[cc]], comp, x, y, z, s.scale);
      out += s.wt[cc] * val;
      H[0] += d.dW[0][cc] * val;
      H[1] += d.dW[1][cc] * val;
      H[2] += d.dW[2][cc] * val;
      if (q_passes(D.g, D.ph, x, y, z, s.scale)) atomicAdd(lamv0 + comp * nc + s.idx[cc], l[comp] * s.wt[cc]);
    }
#pragma unroll
    for (int a = 0; a < 3; a++) gsum[a] += l[comp] * (H[a] - out * d.G[a]) / s.wAcc;
  }
  const float f = -(D.ph.dt * D.ph.rdx) / (float)s.scale;
#pragma unroll
  for (int a = 0; a < 3; a++) atomicAdd(lamv0 + a * nc + cell, f * gsum[a]);
}

// Pressure-gradient transpose: v_a -= alpha (w_R (p_R - p) + w_L (p - p_L))
// on leaf cells; lamP += d v_a / d p times the adjoint of v_a.
__global__ void __launch_bounds__(256) k_adj_gradient(Dev D, const float *lamv, float *lamP, size_t nc) {
  const long long b = adj_block();
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  const float alpha = 0.5f * D.ph.rdx / (float)(1 << bp.w);
  for (int a = 0; a < 3; a++) {
    const float l = lamv[a * nc + cell];
    if (l == 0.f) continue;
    const size_t L = apron_cell(D, (uint32_t)b, bp, ax - (a == 0), ay - (a == 1), az - (a == 2));
    const size_t R = apron_cell(D, (uint32_t)b, bp, ax + (a == 0), ay + (a == 1), az + (a == 2));
    const float wL = D.w[L], wR = D.w[R];
    atomicAdd(lamP + R, -alpha * wR * l);
    atomicAdd(lamP + cell, -alpha * (wL - wR) * l);
    atomicAdd(lamP + L, alpha * wL * l);
  }
}

// One Jacobi sweep of `level` transposed: the sweep wrote dst = (sum of the
// six src neighbours - alpha div) / 6 on the level's cells; its adjoint moves
// lam_dst of each cell (then zero: the overwritten value is dead) to the
// neighbours' lam_src and to lam_div.
__global__ void __launch_bounds__(256) k_adj_jacobi(Dev D, int level, float *lam_dst, float *lam_src,
                                                    float *lam_div) {
  const long long sl = adj_block();
  if (sl >= D.g.budget[level]) return;
  const long long b = D.g.off[level] + sl;
  if (D.pos[b].w != level) return;
  const size_t cell = (size_t)b * BV + (threadIdx.x & 63);
  const float l = lam_dst[cell];
  if (l == 0.f) return;
  lam_dst[cell] = 0.f;
  const Nb6 n = jacobi_neighbours(D, (long long)cell);
  const float l6 = l / 6.f;
  atomicAdd(lam_src + n.i0, l6);
  atomicAdd(lam_src + n.i1, l6);
  atomicAdd(lam_src + n.i2, l6);
  atomicAdd(lam_src + n.i3, l6);
  atomicAdd(lam_src + n.i4, l6);
  atomicAdd(lam_src + n.i5, l6);
  const int s = 1 << level;
  const float alpha = (float)(s * s) * D.ph.dx * D.ph.dx;
  lam_div[cell] += -alpha * l6;
}

// Prolongation transpose of `level`: the level's initial pressure (lam0 of
// its cells, then zero) goes to the parent's apron cells with the 27/9/3/1
// weights of prolong_cell.
__global__ void __launch_bounds__(256) k_adj_prolong(Dev D, int level, float *lam0) {
  const long long sl = adj_block();
  if (sl >= D.g.budget[level]) return;
  const uint32_t b = (uint32_t)(D.g.off[level] + sl);
  const int4 bp = D.pos[b];
  if (bp.w != level) return;
  const uint32_t par = D.parent[b];
  if (par == NONE) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  const float l = lam0[cell];
  lam0[cell] = 0.f;
  if (l == 0.f) return;
  const uint32_t pb = par >> 3;
  const int4 pbp = D.pos[pb];
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz;
  const int ax = 1 + (x / 2) % BW, ay = 1 + (y / 2) % BW, az = 1 + (z / 2) % BW;
  const int i = x % 2 ? 1 : -1, j = y % 2 ? 1 : -1, k = z % 2 ? 1 : -1;
  const float l64 = l / 64.f;
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax, ay, az), 27.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax, ay, az + k), 9.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax, ay + j, az), 9.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax + i, ay, az), 9.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax, ay + j, az + k), 3.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax + i, ay, az + k), 3.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax + i, ay + j, az), 3.f * l64);
  atomicAdd(lam0 + apron_cell(D, pb, pbp, ax + i, ay + j, az + k), 1.f * l64);
}

// Divergence transpose: div = alpha * sum of +-w_n v_n over the six
// neighbours (boundary values replaced by the velocity boundary condition)
// on leaf cells; lamv += d div / d v_n times the adjoint of div where the
// boundary condition passes the neighbour's value through.
__global__ void __launch_bounds__(256) k_adj_divergence(Dev D, const float *lamd, float *lamv, size_t nc) {
  const long long b = adj_block();
  if (b >= D.g.B) return;
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  const int c = threadIdx.x & 63;
  const size_t cell = (size_t)b * BV + c;
  if (D.child[cell >> 3] != NONE) return;
  const float l = lamd[cell];
  if (l == 0.f) return;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  const int scale = 1 << bp.w;
  const float alpha = 0.5f * D.ph.rdx / (float)scale;
  const int x = bp.x + lx, y = bp.y + ly, z = bp.z + lz;
  for (int a = 0; a < 3; a++)
    for (int sgn = -1; sgn <= 1; sgn += 2) {
      const int da = a == 0 ? sgn : 0, db = a == 1 ? sgn : 0, dc = a == 2 ? sgn : 0;
      if (!q_passes(D.g, D.ph, x + da, y + db, z + dc, scale)) continue;
      const size_t n = apron_cell(D, (uint32_t)b, bp, ax + da, ay + db, az + dc);
      atomicAdd(lamv + a * nc + n, (float)sgn * alpha * D.w[n] * l);
    }
}

static unsigned adj_grid(long long blocks) { return (unsigned)((blocks + 3) / 4); }
static void adj_restrict_all(const Dev &D, float *lam, cudaStream_t st) {
  for (int level = D.g.levels - 2; level >= 0; level--) {
    const long long n = 8 * D.g.budget[level];
    k_adj_restrict<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(D, level, lam);
  }
}
static void adj_propagate_all(const Dev &D, float *lam, int sms, cudaStream_t st) {
  const unsigned gs = (unsigned)(sms > 0 ? sms * 4 : 512);
  for (int level = 0; level <= D.g.levels - 2; level++) k_adj_propagate<<<gs, 256, 0, st>>>(D, level, lam);
}

void launch_adjoint_full_phase_a(const Dev &DA, const AdjFull &A, float *lam_em, int sweeps, int sms,
                                 cudaStream_t st) {
  const size_t nc = (size_t)DA.g.B * BV;
  const int nq = DA.g.nq;
  // scalar advection (after the projection): restriction^T, then the scatter
  // into lam_q (the scalars before their advection) and the position part
  // into lam_v (the projected velocity)
  for (int k = 0; k < nq; k++) adj_restrict_all(DA, A.lq + k * nc, st);
  cudaMemsetAsync(A.out_q, 0, nq * nc * sizeof(float), st);
  k_adj_scalars_full<<<adj_grid(DA.g.B), 256, 0, st>>>(DA, A.lq, A.out_q, A.lv, lam_em, nc);
  // projection: restriction^T of the projected velocity, gradient^T into
  // the pressure, the cascade transposed, restriction^T of the divergence,
  // divergence^T back into the velocity
  for (int d = 0; d < 3; d++) adj_restrict_all(DA, A.lv + d * nc, st);
  cudaMemsetAsync(A.lp0, 0, 3 * nc * sizeof(float), st);  // lp0, lp1, ld
  k_adj_gradient<<<adj_grid(DA.g.B), 256, 0, st>>>(DA, A.lv, A.lp0, nc);
  const int top = DA.g.levels - 1;
  for (int level = 0; level <= top; level++) {
    const unsigned g = adj_grid(DA.g.budget[level]);
    for (int it = sweeps - 1; it >= 0; it--) {
      // sweep it read src = (it odd ? p~ : p) and wrote dst = the other plane
      float *ldst = (it & 1) ? A.lp0 : A.lp1, *lsrc = (it & 1) ? A.lp1 : A.lp0;
      k_adj_jacobi<<<g, 256, 0, st>>>(DA, level, ldst, lsrc, A.ld);
    }
    if (level < top) k_adj_prolong<<<g, 256, 0, st>>>(DA, level, A.lp0);
  }
  adj_restrict_all(DA, A.ld, st);
  k_adj_divergence<<<adj_grid(DA.g.B), 256, 0, st>>>(DA, A.ld, A.lv, nc);
  // propagation into the blocks the adaptation moved or created
  for (int d = 0; d < 3; d++) adj_propagate_all(DA, A.lv + d * nc, sms, st);
  for (int k = 0; k < nq; k++) adj_propagate_all(DA, A.out_q + k * nc, sms, st);
}

void launch_adjoint_full_phase_b(const Dev &D0, const AdjFull &A, cudaStream_t st) {
  const size_t nc = (size_t)D0.g.B * BV;
  for (int d = 0; d < 3; d++) adj_restrict_all(D0, A.lv + d * nc, st);
  cudaMemsetAsync(A.out_v, 0, 3 * nc * sizeof(float), st);
  k_adj_velocity_full<<<adj_grid(D0.g.B), 256, 0, st>>>(D0, A.lv, A.out_v, A.out_q, nc);
}

}  // namespace dcg
