// k_uniform.cu — the uniform-grid step (the reference's FluidSimulationUniform,
// src/uniformgrid/*.cu): dense x-fastest fields with a mip-mapped
// pressure / divergence / fluidity pyramid. One thread per cell, linear index
// with x fastest, so every warp reads 128 contiguous bytes of each field.
#include "dcg_kernels.h"

namespace dcg {

__device__ inline size_t uidx(const UDev &U, int x, int y, int z) {
  return ((size_t)z * U.gy + y) * U.gx + x;
}
// mipmapIdx (src/utils/grid_math.cuh:41-52)
__device__ inline size_t umip(const UDev &U, int x, int y, int z, int level) {
  const int s = 1 << level;
  return (size_t)U.mip_off[level] + ((size_t)z * (U.gy / s) + y) * (U.gx / s) + x;
}

// k_uniform_set_solidity_ratio (uniformgrid_structure.cu:23-31)
__global__ void __launch_bounds__(256) k_u_fluidity(UDev U, int level) {
  const int s = 1 << level;
  const long long n = (long long)(U.gx / s) * (U.gy / s) * (U.gz / s);
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int w = U.gx / s, h = U.gy / s;
  const int x = (int)(i % w), y = (int)((i / w) % h), z = (int)(i / ((long long)w * h));
  U.w[umip(U, x, y, z, level)] = fluidity(U.g, U.ph, x, y, z, s);
}

__global__ void __launch_bounds__(256) k_u_sources(UDev U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= U.nc) return;
  const int x = (int)(i % U.gx), y = (int)((i / U.gx) % U.gy), z = (int)(i / ((long long)U.gx * U.gy));
  if (in_source(U.ph, x, y, z, 1))
    for (int k = 0; k < U.nq; k++) U.q[k][i] = src_value_at(U.ph, k, x, y, z, 0);
}

struct USmp {
  size_t idx[8];
  float wt[8];
  float wAcc;
  int x0, y0, z0, x1, y1, z1;
};
// INIT_SAMPLE (uniformgrid_fluid.cu:7-48)
__device__ inline void u_sample(const UDev &U, float px, float py, float pz, USmp &s) {
  const float x = px - 0.5f, y = py - 0.5f, z = pz - 0.5f;
  const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
  s.x0 = (int)xf; s.y0 = (int)yf; s.z0 = (int)zf;
  s.x1 = s.x0 + 1; s.y1 = s.y0 + 1; s.z1 = s.z0 + 1;
  const int x0c = clampi(s.x0, 0, U.gx - 1), y0c = clampi(s.y0, 0, U.gy - 1), z0c = clampi(s.z0, 0, U.gz - 1);
  const int x1c = clampi(s.x1, 0, U.gx - 1), y1c = clampi(s.y1, 0, U.gy - 1), z1c = clampi(s.z1, 0, U.gz - 1);
  s.idx[0] = uidx(U, x0c, y0c, z0c); s.idx[1] = uidx(U, x0c, y0c, z1c);
  s.idx[2] = uidx(U, x0c, y1c, z0c); s.idx[3] = uidx(U, x0c, y1c, z1c);
  s.idx[4] = uidx(U, x1c, y0c, z0c); s.idx[5] = uidx(U, x1c, y0c, z1c);
  s.idx[6] = uidx(U, x1c, y1c, z0c); s.idx[7] = uidx(U, x1c, y1c, z1c);
  const float dx = x - xf, dy = y - yf, dz = z - zf;
  const float Dx = 1.f - dx, Dy = 1.f - dy, Dz = 1.f - dz;
  s.wt[0] = U.w[s.idx[0]] * Dx * Dy * Dz;
  s.wt[1] = U.w[s.idx[1]] * Dx * Dy * dz;
  s.wt[2] = U.w[s.idx[2]] * Dx * dy * Dz;
  s.wt[3] = U.w[s.idx[3]] * Dx * dy * dz;
  s.wt[4] = U.w[s.idx[4]] * dx * Dy * Dz;
  s.wt[5] = U.w[s.idx[5]] * dx * Dy * dz;
  s.wt[6] = U.w[s.idx[6]] * dx * dy * Dz;
  s.wt[7] = U.w[s.idx[7]] * dx * dy * dz;
  s.wAcc = s.wt[0] + s.wt[1] + s.wt[2] + s.wt[3] + s.wt[4] + s.wt[5] + s.wt[6] + s.wt[7];
  const float wInv = 1.f / s.wAcc;
#pragma unroll
  for (int c = 0; c < 8; c++) s.wt[c] = s.wt[c] * wInv;
}

// k_uniform_advect_velocity (uniformgrid_fluid.cu:88-96) + buoyancy extension
__global__ void __launch_bounds__(256) k_u_advect_velocity(UDev U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= U.nc) return;
  const int x = (int)(i % U.gx), y = (int)((i / U.gx) % U.gy), z = (int)(i / ((long long)U.gx * U.gy));
  const float px = ((float)x + 0.5f) - U.v[0][i] * U.ph.dt * U.ph.rdx;
  const float py = ((float)y + 0.5f) - U.v[1][i] * U.ph.dt * U.ph.rdx;
  const float pz = ((float)z + 0.5f) - U.v[2][i] * U.ph.dt * U.ph.rdx;
  USmp s;
  u_sample(U, px, py, pz, s);
  float o0 = 0.f, o1 = 0.f, o2 = 0.f;
  if (!(s.wAcc < 1e-6f)) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int cx = (c & 4) ? s.x1 : s.x0, cy = (c & 2) ? s.y1 : s.y0, cz = (c & 1) ? s.z1 : s.z0;
      float vx = U.v[0][s.idx[c]], vy = U.v[1][s.idx[c]], vz = U.v[2][s.idx[c]];
      vel_bc(U.g, U.ph, vx, vy, vz, cx, cy, cz, 1);
      if (c == 0) {
        o0 = vx * s.wt[0]; o1 = vy * s.wt[0]; o2 = vz * s.wt[0];
      } else {
        o0 = o0 + vx * s.wt[c]; o1 = o1 + vy * s.wt[c]; o2 = o2 + vz * s.wt[c];
      }
    }
  }
  if (U.ph.buoy_a != 0.f || U.ph.buoy_b != 0.f) {
    float f = -U.ph.buoy_a * U.q[0][i];
    if (U.nq > 1) f = f + U.ph.buoy_b * (U.q[1][i] - U.ph.t_amb);
    o1 = o1 + U.ph.dt * f;
  }
  U.tv[0][i] = o0;
  U.tv[1][i] = o1;
  U.tv[2][i] = o2;
}

// k_uniform_advect_density (uniformgrid_fluid.cu:98-105) + sources
__global__ void __launch_bounds__(256) k_u_advect_scalars(UDev U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= U.nc) return;
  const int x = (int)(i % U.gx), y = (int)((i / U.gx) % U.gy), z = (int)(i / ((long long)U.gx * U.gy));
  const float px = ((float)x + 0.5f) - U.v[0][i] * U.ph.dt * U.ph.rdx;
  const float py = ((float)y + 0.5f) - U.v[1][i] * U.ph.dt * U.ph.rdx;
  const float pz = ((float)z + 0.5f) - U.v[2][i] * U.ph.dt * U.ph.rdx;
  USmp s;
  u_sample(U, px, py, pz, s);
  const bool src = in_source(U.ph, x, y, z, 1);
  for (int k = 0; k < U.nq; k++) {
    float acc = 0.f;
    if (!(s.wAcc < 1e-6f)) {
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int cx = (c & 4) ? s.x1 : s.x0, cy = (c & 2) ? s.y1 : s.y0, cz = (c & 1) ? s.z1 : s.z0;
        const float qc = q_bc(U.g, U.ph, U.q[k][s.idx[c]], k, cx, cy, cz, 1);
        acc = (c == 0) ? qc * s.wt[0] : acc + qc * s.wt[c];
      }
    }
    if (k == 0 && U.ph.em_n > 0) acc = acc + U.ph.dt * emission_at(U.g, U.ph, x, y, z, 1);
    U.tq[k][i] = src ? src_value_at(U.ph, k, x, y, z, 0) : acc;
  }
}

// k_uniform_calc_divergence (uniformgrid_fluid.cu:107-132)
__global__ void __launch_bounds__(256) k_u_divergence(UDev U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= U.nc) return;
  const int gx = U.gx, gy = U.gy, gz = U.gz;
  const int x = (int)(i % gx), y = (int)((i / gx) % gy), z = (int)(i / ((long long)gx * gy));
  const size_t il = x > 0 ? i - 1 : i, ir = x < gx - 1 ? i + 1 : i;
  const size_t id = y > 0 ? i - gx : i, iu = y < gy - 1 ? i + gx : i;
  const size_t ib = z > 0 ? i - (size_t)gx * gy : i, iff = z < gz - 1 ? i + (size_t)gx * gy : i;
  U.p[i] = 0.f;
  U.pt[i] = 0.f;
  float a0, a1, a2;
  float vl, vr, vd, vu, vb, vf;
  a0 = U.v[0][il]; a1 = U.v[1][il]; a2 = U.v[2][il]; vel_bc(U.g, U.ph, a0, a1, a2, x - 1, y, z, 1); vl = a0;
  a0 = U.v[0][ir]; a1 = U.v[1][ir]; a2 = U.v[2][ir]; vel_bc(U.g, U.ph, a0, a1, a2, x + 1, y, z, 1); vr = a0;
  a0 = U.v[0][id]; a1 = U.v[1][id]; a2 = U.v[2][id]; vel_bc(U.g, U.ph, a0, a1, a2, x, y - 1, z, 1); vd = a1;
  a0 = U.v[0][iu]; a1 = U.v[1][iu]; a2 = U.v[2][iu]; vel_bc(U.g, U.ph, a0, a1, a2, x, y + 1, z, 1); vu = a1;
  a0 = U.v[0][ib]; a1 = U.v[1][ib]; a2 = U.v[2][ib]; vel_bc(U.g, U.ph, a0, a1, a2, x, y, z - 1, 1); vb = a2;
  a0 = U.v[0][iff]; a1 = U.v[1][iff]; a2 = U.v[2][iff]; vel_bc(U.g, U.ph, a0, a1, a2, x, y, z + 1, 1); vf = a2;
  const float *W = U.w;
  U.div[i] = 0.5f * U.ph.rdx * (W[ir] * vr - W[il] * vl + W[iu] * vu - W[id] * vd + W[iff] * vf - W[ib] * vb);
}

// k_uniform_restrict (uniformgrid_fluid.cu:134-160)
__global__ void __launch_bounds__(256) k_u_restrict(UDev U, int level) {
  const int s = 1 << level, cs = s / 2;
  const int w = U.gx / s, h = U.gy / s, d = U.gz / s;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)w * h * d) return;
  const int x = (int)(i % w), y = (int)((i / w) % h), z = (int)(i / ((long long)w * h));
  const int wc = U.gx / cs, hc = U.gy / cs;
  const size_t idx = umip(U, x, y, z, level);
  const size_t i000 = umip(U, 2 * x, 2 * y, 2 * z, level - 1);
  const size_t i001 = i000 + 1, i010 = i000 + wc, i011 = i010 + 1;
  const size_t i100 = i000 + (size_t)wc * hc, i101 = i100 + 1, i110 = i100 + wc, i111 = i110 + 1;
  U.p[idx] = 0.f;
  U.pt[idx] = 0.f;
  const float *V = U.div;
  U.div[idx] = 0.125f * (V[i000] + V[i001] + V[i010] + V[i011] + V[i100] + V[i101] + V[i110] + V[i111]);
}

// calcPressure / k_uniform_jacobi(_inv) (uniformgrid_fluid.cu:162-204)
__global__ void __launch_bounds__(256) k_u_jacobi(UDev U, int level, const float *__restrict__ src,
                                                  float *__restrict__ dst) {
  const int s = 1 << level;
  const int w = U.gx / s, h = U.gy / s, d = U.gz / s;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)w * h * d) return;
  const int x = (int)(i % w), y = (int)((i / w) % h), z = (int)(i / ((long long)w * h));
  const size_t idx = (size_t)U.mip_off[level] + (size_t)i;
  const size_t il = x > 0 ? idx - 1 : idx, ir = x < w - 1 ? idx + 1 : idx;
  const size_t id = y > 0 ? idx - w : idx, iu = y < h - 1 ? idx + w : idx;
  const size_t ib = z > 0 ? idx - (size_t)w * h : idx, iff = z < d - 1 ? idx + (size_t)w * h : idx;
  const float alpha = U.ph.dx * U.ph.dx * (float)s * (float)s;
  dst[idx] = div6(src[il] + src[ir] + src[id] + src[iu] + src[ib] + src[iff] - alpha * U.div[idx]);
}

// k_uniform_prolongate (uniformgrid_fluid.cu:206-237)
__global__ void __launch_bounds__(256) k_u_prolongate(UDev U, int level) {
  const int s = 1 << level;
  const int w = U.gx / s, h = U.gy / s, d = U.gz / s;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)w * h * d) return;
  const int x = (int)(i % w), y = (int)((i / w) % h), z = (int)(i / ((long long)w * h));
  const size_t idx = (size_t)U.mip_off[level] + (size_t)i;
  const size_t i000 = umip(U, x / 2, y / 2, z / 2, level + 1);
  const int sx = (x == 0 || x == w - 1) ? 0 : 2 * (x % 2) - 1;
  const int sy = (y == 0 || y == h - 1) ? 0 : 2 * (y % 2) - 1;
  const int sz = (z == 0 || z == d - 1) ? 0 : 2 * (z % 2) - 1;
  const size_t i001 = i000 + sx;
  const size_t i010 = i000 + (long long)sy * w / 2;
  const size_t i011 = i010 + sx;
  const size_t i100 = i000 + (long long)sz * (w / 2) * (h / 2);
  const size_t i101 = i100 + sx;
  const size_t i110 = i100 + (long long)sy * (w / 2);
  const size_t i111 = i110 + sx;
  const float *P = U.p;
  U.p[idx] = (27.f * P[i000] + 9.f * (P[i001] + P[i010] + P[i100]) + 3.f * (P[i011] + P[i101] + P[i110]) +
              P[i111]) / 64.f;
}

// k_uniform_apply_pressure (uniformgrid_fluid.cu:239-260)
__global__ void __launch_bounds__(256) k_u_apply_pressure(UDev U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= U.nc) return;
  const int gx = U.gx, gy = U.gy, gz = U.gz;
  const int x = (int)(i % gx), y = (int)((i / gx) % gy), z = (int)(i / ((long long)gx * gy));
  const size_t il = x > 0 ? i - 1 : i, ir = x < gx - 1 ? i + 1 : i;
  const size_t id = y > 0 ? i - gx : i, iu = y < gy - 1 ? i + gx : i;
  const size_t ib = z > 0 ? i - (size_t)gx * gy : i, iff = z < gz - 1 ? i + (size_t)gx * gy : i;
  const float alpha = 0.5f * U.ph.rdx;
  const float *P = U.p, *W = U.w;
  const float pc = P[i];
  U.v[0][i] = U.v[0][i] - alpha * (W[ir] * (P[ir] - pc) + W[il] * (pc - P[il]));
  U.v[1][i] = U.v[1][i] - alpha * (W[iu] * (P[iu] - pc) + W[id] * (pc - P[id]));
  U.v[2][i] = U.v[2][i] - alpha * (W[iff] * (P[iff] - pc) + W[ib] * (pc - P[ib]));
}

__global__ void __launch_bounds__(256) k_u_noise(UDev U, unsigned long long seed, float amp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= U.nc) return;
  const int x = (int)(i % U.gx), y = (int)((i / U.gx) % U.gy), z = (int)(i / ((long long)U.gx * U.gy));
  for (int d = 0; d < 3; d++) U.v[d][i] = U.v[d][i] + amp * noise_unit(seed, x, y, z, 0, d);
}

// k_uniform_debug_stats (uniformgrid_structure.cu:33-43): sum rho * w.
__global__ void __launch_bounds__(256) k_u_stats(UDev U) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (i < U.nc) m = (double)U.q[0][i] * (double)U.w[i];
  for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
  if ((threadIdx.x & 31) == 0 && m != 0.0) atomicAdd(&U.red[1], m);
}

static unsigned ugrid(long long n) { return (unsigned)((n + 255) / 256); }
static long long ucells(const UDev &U, int level) {
  const int s = 1 << level;
  return (long long)(U.gx / s) * (U.gy / s) * (U.gz / s);
}

void launch_u_fluidity(const UDev &U, cudaStream_t st) {
  for (int l = 0; l < U.levels; l++) k_u_fluidity<<<ugrid(ucells(U, l)), 256, 0, st>>>(U, l);
}
void launch_u_sources(const UDev &U, cudaStream_t st) { k_u_sources<<<ugrid(U.nc), 256, 0, st>>>(U); }
void launch_u_advect_velocity(const UDev &U, cudaStream_t st) {
  k_u_advect_velocity<<<ugrid(U.nc), 256, 0, st>>>(U);
}
void launch_u_advect_scalars(const UDev &U, cudaStream_t st) {
  k_u_advect_scalars<<<ugrid(U.nc), 256, 0, st>>>(U);
}
// FluidSimulationUniform::project / projectLocal (fluid_simulation_uniform.cu:96-135)
void launch_u_project(const UDev &U, int top_pairs, int pairs, bool local, cudaStream_t st) {
  k_u_divergence<<<ugrid(U.nc), 256, 0, st>>>(U);
  if (local) {
    for (int i = 0; i < pairs; i++) {
      k_u_jacobi<<<ugrid(U.nc), 256, 0, st>>>(U, 0, U.p, U.pt);
      k_u_jacobi<<<ugrid(U.nc), 256, 0, st>>>(U, 0, U.pt, U.p);
    }
  } else {
    for (int l = 1; l < U.levels; l++) k_u_restrict<<<ugrid(ucells(U, l)), 256, 0, st>>>(U, l);
    const int top = U.levels - 1;
    for (int i = 0; i < top_pairs; i++) {
      k_u_jacobi<<<ugrid(ucells(U, top)), 256, 0, st>>>(U, top, U.p, U.pt);
      k_u_jacobi<<<ugrid(ucells(U, top)), 256, 0, st>>>(U, top, U.pt, U.p);
    }
    for (int l = U.levels - 2; l >= 0; l--) {
      k_u_prolongate<<<ugrid(ucells(U, l)), 256, 0, st>>>(U, l);
      for (int i = 0; i < pairs; i++) {
        k_u_jacobi<<<ugrid(ucells(U, l)), 256, 0, st>>>(U, l, U.p, U.pt);
        k_u_jacobi<<<ugrid(ucells(U, l)), 256, 0, st>>>(U, l, U.pt, U.p);
      }
    }
  }
  k_u_apply_pressure<<<ugrid(U.nc), 256, 0, st>>>(U);
}
void launch_u_add_noise(const UDev &U, unsigned long long seed, float amp, cudaStream_t st) {
  k_u_noise<<<ugrid(U.nc), 256, 0, st>>>(U, seed, amp);
}
void launch_u_stats(const UDev &U, cudaStream_t st) {
  cudaMemsetAsync(U.red, 0, sizeof(double) * 32, st);
  k_u_stats<<<ugrid(U.nc), 256, 0, st>>>(U);
}

}  // namespace dcg
