// dcg_oracle.cpp — CPU oracle of the DCGrid simulation step (TEST INFRASTRUCTURE).
//
// A plain C++ restatement of the reference's adaptive-grid and uniform-grid
// simulation steps. Each function names the reference file:line it follows.
// Field arithmetic is templated: R = float reproduces the reference's FP32
// operation order (build with -ffp-contract=off), R = double is the FP64
// oracle. Topology scores are always float, as in the reference.
//
// Only tests, the smoke check and the CPU-baseline leg of the benchmark use
// this library; the product never links it.
#include "dcg_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int BW = 4;    // DCGrid::blockW   (src/dcgrid/dcgrid.h:52)
constexpr int BV = 64;   // DCGrid::blockV
constexpr int AW = 6;    // DCGrid::apronW
constexpr int AA = 36;   // DCGrid::apronA
constexpr int AV = 216;  // DCGrid::apronV
constexpr int64_t NF = -1;  // DCGrid::notFound
constexpr uint8_t FREE = 0xFF;
constexpr uint8_t MOVED = 1, REFINED = 2;  // dcgrid.h:45-49

// iDivUp (src/utils/grid_math.cuh:5-7)
inline int idiv_up(int a, int b) { return (a % b != 0) ? (a / b + 1) : (a / b); }

// bitSpread3 / gridHash (src/dcgrid/dcgrid_utils.cuh:83-96)
inline uint32_t bit_spread3(uint32_t data) {
  uint32_t res = 0;
  for (uint32_t mask = 1u; mask; mask <<= 3, data <<= 2) res |= data & mask;
  return res;
}
inline uint32_t grid_hash(int x, int y, int z) {
  return (bit_spread3((uint32_t)(x / BW)) << 2) |
         (bit_spread3((uint32_t)(y / BW)) << 1) | bit_spread3((uint32_t)(z / BW));
}

// SPREAD (dcgrid_utils.cuh:67): local coordinate -> local cell index bits.
inline int spread(int d, int off) { return ((d & 1) | ((d << 2) & 8)) << off; }
inline int local_of(int x, int y, int z) {
  return spread(x, 2) + spread(y, 1) + spread(z, 0);
}
// IDX2POS (dcgrid_utils.cuh:69-72): local cell index -> local coordinates.
inline void local_xyz(int c, int &x, int &y, int &z) {
  const int sub = c >> 3;
  x = (((sub >> 2) & 1) << 1) | ((c >> 2) & 1);
  y = (((sub >> 1) & 1) << 1) | ((c >> 1) & 1);
  z = ((sub & 1) << 1) | (c & 1);
}
inline int clampi(int v, int a, int b) { return v < a ? a : (v > b ? b : v); }

template <typename R> inline R clampr(R v, R a, R b) {
  return v < a ? a : (v > b ? b : v);
}

// 16-bit storage of the advected scalars (DCG_PRECISION_MIXED*): the value is
// rounded to nearest even in BF16 (1) or FP16 (2) and widened back.
inline float round_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return f;  // inf / nan unchanged
  u += 0x7FFFu + ((u >> 16) & 1u);
  u &= 0xFFFF0000u;
  std::memcpy(&f, &u, 4);
  return f;
}
inline float round_fp16(float f) { return (float)(_Float16)f; }
template <typename R> inline R store_q(R v, int precision) {
  if (precision == DCG_PRECISION_MIXED) return (R)round_bf16((float)v);
  if (precision == DCG_PRECISION_MIXED_FP16) return (R)round_fp16((float)v);
  return v;
}

// Seeded value noise used by the terrain extension. Lattice values come from
// a 32-bit integer hash; (h >> 8) * 2^-24 is exact in float and double.
inline uint32_t hash32(uint32_t seed, int32_t i, int32_t k, int32_t o) {
  uint32_t h = seed ^ 0x9E3779B9u;
  h ^= (uint32_t)i * 0x85EBCA6Bu; h = (h ^ (h >> 15)) * 0x2C1B3C6Du;
  h ^= (uint32_t)k * 0xC2B2AE35u; h = (h ^ (h >> 13)) * 0x297A2D39u;
  h ^= (uint32_t)o * 0x27D4EB2Fu; h = (h ^ (h >> 16)) * 0x85EBCA77u;
  return h ^ (h >> 15);
}

// splitmix64 finaliser, used for the seeded velocity noise.
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline float noise_unit(uint64_t seed, int x, int y, int z, int level, int comp) {
  uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(comp + 1));
  h = mix64(h ^ ((uint64_t)(uint32_t)x * 0xD6E8FEB86659FD93ull));
  h = mix64(h ^ ((uint64_t)(uint32_t)y * 0xA0761D6478BD642Full));
  h = mix64(h ^ ((uint64_t)(uint32_t)z * 0xE7037ED1A0B428DBull));
  h = mix64(h ^ (uint64_t)(uint32_t)level);
  const float u = (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
  return 2.0f * u - 1.0f;
}

struct Base {
  dcg_params P{};
  float rdx_f = 1.f;
  std::string err;
  int mode = 0;
  int prec = 0;
  int64_t steps = 0;
  virtual ~Base() {}
  virtual int reset() = 0;
  virtual int advect_velocity() = 0;
  virtual int adapt() = 0;
  virtual int project() = 0;
  virtual int project_local() = 0;
  virtual int advect_scalars() = 0;
  virtual int add_noise(uint64_t seed, float amp) = 0;
  virtual void info(dcg_info *i) const = 0;
  virtual int get_field(int f, double *dst) = 0;
  virtual int set_field(int f, const double *src) = 0;
  virtual int get_dense(int f, double *dst) = 0;
  virtual int stats(dcg_stats *st) = 0;
  virtual int set_emission(const double *src) = 0;
  virtual int render(const dcg_render_params &rp, double *out) const = 0;
  // dcg_set_heightmap: replaces the noise terrain (empty map: back to it) and resets
  virtual int set_heightmap(const float *h, int nx, int nz) = 0;
  std::vector<float> hmap;
  int store_heightmap(const float *h, int nx, int nz) {
    if (h && (nx <= 0 || nz <= 0 || nx > 65536 || nz > 65536 || (int64_t)nx * nz > (1ll << 27)))
      return fail(DCG_E_INVALID, "heightmap: 1 <= nx, nz <= 65536 and nx * nz <= 2^27");
    if (!h && (nx != 0 || nz != 0)) return fail(DCG_E_INVALID, "heightmap: no heights given for nx, nz > 0");
    if (h) hmap.assign(h, h + (size_t)nx * nz);
    else hmap.clear();
    return DCG_OK;
  }
  int fail(int code, const char *msg) {
    err = msg;
    return code;
  }
  // Step order of Simulation::updateSimulation (src/simulation.cpp:104-112).
  int step(int n) {
    for (int i = 0; i < n; i++) {
      int rc;
      if ((rc = advect_velocity())) return rc;
      if ((rc = adapt())) return rc;
      if ((rc = project())) return rc;
      if ((rc = advect_scalars())) return rc;
      steps++;
    }
    return DCG_OK;
  }
};

// Physics shared by both grid types: boundary conditions, fluidity, sources.
template <typename R> struct Physics {
  const dcg_params *P;
  R rdx, dt, dx;
  int gx, gy, gz;
  // terrain heightmap (extension, dcg_set_heightmap): nx*nz texels, x fastest
  const float *hm = nullptr;
  int hm_nx = 0, hm_nz = 0;
  R hm_sx = 0, hm_sz = 0;  // texels per finest cell

  // Bilinear sample at (x, z), texel centres at (i + 0.5) / hm_sx, edge
  // texels extended; the coordinate is clamped to [-1, n] first (fmax/fmin:
  // a NaN coordinate becomes -1).
  R heightmap_sample(R x, R z) const {
    const R u = std::fmin(std::fmax(x * hm_sx - (R)0.5f, (R)-1), (R)hm_nx);
    const R v = std::fmin(std::fmax(z * hm_sz - (R)0.5f, (R)-1), (R)hm_nz);
    const R iu = std::floor(u), iv = std::floor(v);
    const R fu = u - iu, fv = v - iv;
    const int i0 = std::min(std::max((int)iu, 0), hm_nx - 1), i1 = std::min(std::max((int)iu + 1, 0), hm_nx - 1);
    const int k0 = std::min(std::max((int)iv, 0), hm_nz - 1), k1 = std::min(std::max((int)iv + 1, 0), hm_nz - 1);
    const R h00 = (R)hm[(size_t)k0 * hm_nx + i0], h10 = (R)hm[(size_t)k0 * hm_nx + i1];
    const R h01 = (R)hm[(size_t)k1 * hm_nx + i0], h11 = (R)hm[(size_t)k1 * hm_nx + i1];
    const R a = h00 + (h10 - h00) * fu;
    const R b = h01 + (h11 - h01) * fu;
    return a + (b - a) * fv;
  }
  void set_heightmap(const std::vector<float> &m, int nx, int nz) {
    hm = m.empty() ? nullptr : m.data();
    hm_nx = hm ? nx : 0;
    hm_nz = hm ? nz : 0;
    hm_sx = hm ? (R)nx / (R)gx : (R)0;
    hm_sz = hm ? (R)nz / (R)gz : (R)0;
  }

  // sphereSDF (src/sdf.cuh:8-20) and the terrain extension y - h(x, z).
  R terrain_height(R x, R z) const {
    if (hm) return (R)P->terrain_base_height + (R)P->terrain_amplitude * heightmap_sample(x, z);
    R sum = 0, amp = 1, norm = 0, f = (R)P->terrain_frequency;
    for (int o = 0; o < P->terrain_octaves; o++) {
      const R u = x * f, v = z * f;
      const R iu = std::floor(u), iv = std::floor(v);
      const R fu = u - iu, fv = v - iv;
      const R su = fu * fu * ((R)3 - (R)2 * fu);
      const R sv = fv * fv * ((R)3 - (R)2 * fv);
      const int i0 = (int)iu, k0 = (int)iv;
      const R unit = (R)(1.0f / 16777216.0f);
      const R a = (R)(hash32(P->terrain_seed, i0, k0, o) >> 8) * unit;
      const R b = (R)(hash32(P->terrain_seed, i0 + 1, k0, o) >> 8) * unit;
      const R c = (R)(hash32(P->terrain_seed, i0, k0 + 1, o) >> 8) * unit;
      const R d = (R)(hash32(P->terrain_seed, i0 + 1, k0 + 1, o) >> 8) * unit;
      const R ab = a + (b - a) * su;
      const R cd = c + (d - c) * su;
      sum = sum + amp * (ab + (cd - ab) * sv);
      norm = norm + amp;
      amp = amp * (R)P->terrain_persistence;
      f = f * (R)2;
    }
    return (R)P->terrain_base_height + (R)P->terrain_amplitude * (sum / norm);
  }
  R scene_sdf(R x, R y, R z) const {
    R d = (R)FLT_MAX;
    if (P->solids & DCG_SOLIDS_SPHERE) {
      const R cx = (R)gx * (R)0.5f, cy = (R)gy * (R)0.45f, cz = (R)gz * (R)0.5f;
      const R r = (R)P->sphere_radius_world * rdx;
      const R ddx = x - cx, ddy = y - cy, ddz = z - cz;
      d = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz) - r;
    }
    if (P->solids & DCG_SOLIDS_TERRAIN) {
      const R t = y - terrain_height(x, z);
      d = std::min(d, t);
    }
    return d;
  }
  // getCellFluidity (src/utils/sim_utils.cu:11-22)
  R fluidity(int x, int y, int z, int scale) const {
    if (P->solids == DCG_SOLIDS_NONE) return (R)1;
    const R s = (R)scale;
    const R d = scene_sdf(((R)x + (R)0.5f) * s, ((R)y + (R)0.5f) * s,
                          ((R)z + (R)0.5f) * s);
    const R overlap = clampr((R)0.5f - d / (s * (R)1.73205f), (R)0, (R)1);
    return (R)1 - overlap;
  }
  bool in_inlet(int x, int y, int z, int scale) const {
    if (!P->inlet_enabled || y >= 0) return false;
    const R a = (R)(x * scale) - (R)0.5f * (R)gx;
    const R b = (R)(z * scale) - (R)0.5f * (R)gz;
    return std::sqrt(a * a + b * b) < (R)P->emission_radius * rdx;
  }
  bool outside(int x, int y, int z, int scale) const {
    return x < 0 || y < 0 || z < 0 || x * scale >= gx || y * scale >= gy ||
           z * scale >= gz;
  }
  bool yz_inside(int y, int z, int scale) const {
    return y >= 0 && z >= 0 && y * scale < gy && z * scale < gz;
  }
  // velocityBndCond (sim_utils.cu:24-39) + the wind extension.
  void vel_bc(R v[3], int x, int y, int z, int scale) const {
    if (in_inlet(x, y, z, scale)) {
      v[0] = 0; v[1] = (R)P->velocity_emission_rate; v[2] = 0;
      return;
    }
    if (P->wind_enabled && yz_inside(y, z, scale)) {
      if (x < 0) { v[0] = (R)P->wind[0]; v[1] = (R)P->wind[1]; v[2] = (R)P->wind[2]; return; }
      if (x * scale >= gx) return;  // zero-gradient outflow
    }
    if (outside(x, y, z, scale)) v[0] = v[1] = v[2] = 0;
  }
  // densityBndCond (sim_utils.cu:41-55) + the wind extension; scalar k>0
  // (temperature, vapor) has no inlet emission.
  R q_bc(R q, int k, int x, int y, int z, int scale) const {
    if (in_inlet(x, y, z, scale)) return k == 0 ? (R)P->density_emission_rate : (R)0;
    if (P->wind_enabled && yz_inside(y, z, scale)) {
      if (x < 0) return 0;
      if (x * scale >= gx) return q;
    }
    if (outside(x, y, z, scale)) return 0;
    return q;
  }
  bool in_source(int x, int y, int z, int scale) const {
    if (!P->src_enabled) return false;
    const R s = (R)scale;
    const R cx = ((R)x + (R)0.5f) * s - (R)P->src_center[0];
    const R cy = ((R)y + (R)0.5f) * s - (R)P->src_center[1];
    const R cz = ((R)z + (R)0.5f) * s - (R)P->src_center[2];
    return cx * cx + cy * cy + cz * cz < (R)P->src_radius * (R)P->src_radius;
  }
  // Emission field (extension): trilinear sample of the n^3 field over the
  // domain's x, z and the bottom emission_band cells in y; 0 outside the band.
  const std::vector<R> *em = nullptr;
  static R lerp(R a, R b, R t) { return a + (b - a) * t; }
  R emission_at(int x, int y, int z, int scale) const {
    const int n = P->emission_n;
    if (n <= 0 || !em || em->empty()) return 0;
    const R s = (R)scale;
    const R yw = ((R)y + (R)0.5f) * s;
    if (!(yw < (R)P->emission_band)) return 0;
    const R xw = ((R)x + (R)0.5f) * s, zw = ((R)z + (R)0.5f) * s;
    const R top = (R)(n - 1);
    const R u = clampr(xw * ((R)n / (R)gx) - (R)0.5f, (R)0, top);
    const R v = clampr(yw * ((R)n / (R)P->emission_band) - (R)0.5f, (R)0, top);
    const R w = clampr(zw * ((R)n / (R)gz) - (R)0.5f, (R)0, top);
    const int i0 = (int)std::floor(u), j0 = (int)std::floor(v), k0 = (int)std::floor(w);
    const int i1 = i0 + 1 < n ? i0 + 1 : n - 1, j1 = j0 + 1 < n ? j0 + 1 : n - 1, k1 = k0 + 1 < n ? k0 + 1 : n - 1;
    const R fu = u - (R)i0, fv = v - (R)j0, fw = w - (R)k0;
    auto at = [&](int i, int j, int k) { return (*em)[((size_t)k * n + j) * n + i]; };
    const R e00 = lerp(at(i0, j0, k0), at(i1, j0, k0), fu);
    const R e10 = lerp(at(i0, j1, k0), at(i1, j1, k0), fu);
    const R e01 = lerp(at(i0, j0, k1), at(i1, j0, k1), fu);
    const R e11 = lerp(at(i0, j1, k1), at(i1, j1, k1), fu);
    return lerp(lerp(e00, e10, fv), lerp(e01, e11, fv), fw);
  }
  // q_bc passes the scalar through (identity) at this corner
  bool q_passes(int x, int y, int z, int scale) const {
    if (in_inlet(x, y, z, scale)) return false;
    if (P->wind_enabled && yz_inside(y, z, scale)) {
      if (x < 0) return false;
      if (x * scale >= gx) return true;
    }
    return !outside(x, y, z, scale);
  }
  // transpose of emission_at: lam_em[i] += g * d(emission)/d(E[i])
  void emission_adjoint(int x, int y, int z, int scale, double g, double *lam_em) const {
    const int n = P->emission_n;
    const R s = (R)scale;
    const R yw = ((R)y + (R)0.5f) * s;
    if (!(yw < (R)P->emission_band)) return;
    const R xw = ((R)x + (R)0.5f) * s, zw = ((R)z + (R)0.5f) * s;
    const R top = (R)(n - 1);
    const R u = clampr(xw * ((R)n / (R)gx) - (R)0.5f, (R)0, top);
    const R v = clampr(yw * ((R)n / (R)P->emission_band) - (R)0.5f, (R)0, top);
    const R w = clampr(zw * ((R)n / (R)gz) - (R)0.5f, (R)0, top);
    const int i0 = (int)std::floor(u), j0 = (int)std::floor(v), k0 = (int)std::floor(w);
    const int I[2] = {i0, i0 + 1 < n ? i0 + 1 : n - 1}, J[2] = {j0, j0 + 1 < n ? j0 + 1 : n - 1},
              K[2] = {k0, k0 + 1 < n ? k0 + 1 : n - 1};
    const double fu = (double)(u - (R)i0), fv = (double)(v - (R)j0), fw = (double)(w - (R)k0);
    const double WU[2] = {1 - fu, fu}, WV[2] = {1 - fv, fv}, WW[2] = {1 - fw, fw};
    for (int c = 0; c < 8; c++) {
      const int a = (c >> 2) & 1, bb = (c >> 1) & 1, cc = c & 1;
      lam_em[((size_t)K[cc] * n + J[bb]) * n + I[a]] += g * WU[a] * WV[bb] * WW[cc];
    }
  }
  // a source cell's value for scalar k: the temperature with the seeded
  // per-cell jitter of the cell's level-local position (extension)
  R src_value_at(int k, int x, int y, int z, int level) const {
    if (k != 1 || P->src_jitter == 0.f) return src_value(k);
    return (R)(P->src_temperature + P->src_jitter * noise_unit(P->src_jitter_seed, x, y, z, level, 7));
  }
  R src_value(int k) const {
    return k == 0 ? (R)P->src_density : (k == 1 ? (R)P->src_temperature : (R)P->src_vapor);
  }
};

// ======================================================================
//  Ray marcher (src/raymarching.cuh:17-275, camera of k_dcgrid_render,
//  src/dcgrid/dcgrid_rendering.cu:58-92), templated on the grid's sampler
// ======================================================================
template <typename R> struct V3 {
  R x, y, z;
  V3 operator+(V3 o) const { return {x + o.x, y + o.y, z + o.z}; }
  V3 operator-(V3 o) const { return {x - o.x, y - o.y, z - o.z}; }
  V3 operator*(R s) const { return {x * s, y * s, z * s}; }
  V3 operator/(R s) const { return {x / s, y / s, z / s}; }
};
template <typename R> inline R dot3(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> inline R len3(V3<R> a) { return std::sqrt(dot3(a, a)); }
template <typename R> inline V3<R> normalize3(V3<R> a) { return a * ((R)1 / len3(a)); }
template <typename R> struct March {
  int ix, iy, iz;
  R fx, fy, fz;
  size_t idx[8];
  R density;
};
// MarchAux::interpolate (raymarching.cuh:27-42)
template <typename R, class F> inline R interp(const March<R> &a, F f) {
  const R dxInv = (R)1 - a.fx;
  const R c00 = f(a.idx[0]) * dxInv + f(a.idx[4]) * a.fx;
  const R c01 = f(a.idx[1]) * dxInv + f(a.idx[5]) * a.fx;
  const R c10 = f(a.idx[2]) * dxInv + f(a.idx[6]) * a.fx;
  const R c11 = f(a.idx[3]) * dxInv + f(a.idx[7]) * a.fx;
  const R dyInv = (R)1 - a.fy;
  const R c0 = c00 * dyInv + c10 * a.fy;
  const R c1 = c01 * dyInv + c11 * a.fy;
  return c0 * ((R)1 - a.fz) + c1 * a.fz;
}
template <typename R> inline void mix3(V3<R> src, R srcAlpha, V3<R> &dst, R &dstAlpha) {
  if (srcAlpha > (R)1e-6f) {
    const R impact = ((R)1 - dstAlpha) * srcAlpha;
    dst = (dst * dstAlpha + src * impact) / (dstAlpha + impact);
    dstAlpha += impact;
  }
}
// fmax / fmin (IEEE maxNum / minNum: a NaN operand yields the other one) as
// fmaxf / fminf in the reference: rays with a zero direction component reach
// the box test with inf * 0 = NaN terms
template <typename R, class S> struct Marcher {
  const S &G;
  const Physics<R> &ph;
  const dcg_render_params &rp;
  R sdf(V3<R> p) const { return ph.scene_sdf(p.x, p.y, p.z); }
  V3<R> normal(V3<R> p) const {
    const R e = (R)1e-4f;
    return normalize3(V3<R>{sdf({p.x + e, p.y, p.z}) - sdf({p.x - e, p.y, p.z}),
                            sdf({p.x, p.y + e, p.z}) - sdf({p.x, p.y - e, p.z}),
                            sdf({p.x, p.y, p.z + e}) - sdf({p.x, p.y, p.z - e})});
  }
  bool box_hit(R &dNear, R &dFar, V3<R> o, V3<R> dinv) const {
    const R cx = (R)ph.gx * (R)0.5f, cy = (R)ph.gy * (R)0.5f, cz = (R)ph.gz * (R)0.5f;
    const R nx = dinv.x * (o.x - cx), ny = dinv.y * (o.y - cy), nz = dinv.z * (o.z - cz);
    const R kx = std::fabs(dinv.x) * cx, ky = std::fabs(dinv.y) * cy, kz = std::fabs(dinv.z) * cz;
    dNear = std::fmax(std::fmax(-nx - kx, -ny - ky), -nz - kz);
    dFar = std::fmin(std::fmin(-nx + kx, -ny + ky), -nz + kz);
    return dNear < dFar && dFar > (R)0;
  }
  R alpha_of(R dist, R dens) const { return (R)1 - std::exp(-dist * ph.dx * dens); }
  R light_march(V3<R> origin, V3<R> sun, V3<R> suninv) const {
    R light = 1;
    if (rp.solids && ph.P->solids) {
      R dScene = 0;
      for (int i = 0; i < 100; i++) {
        const R s = sdf(origin + sun * dScene);
        light = std::fmin(light, (s / dScene) / (R)0.06f);
        if (light <= (R)1e-2f) return 0;
        dScene += s;
      }
    }
    if (rp.channel == DCG_RENDER_FLUID) {
      R dNear, dFar;
      if (box_hit(dNear, dFar, origin, suninv)) {
        V3<R> pos = origin;
        if (dNear > (R)0) {
          pos = pos + sun * dNear;
          dFar -= dNear;
        }
        const R step = std::fmax(dFar / (R)100, (R)1e-1f);
        R dens = 0;
        March<R> a;
        for (R d = step; d < dFar && dens < (R)5; d += step) {
          pos = pos + sun * step;
          G.sample(pos, rp.precise != 0, a);
          dens += a.density * ph.dx * step;
        }
        light *= std::exp(-dens);
      }
    }
    return light;
  }
  void march(V3<R> origin, V3<R> dir, V3<R> sun, R out[4]) const {
    const R ambient = (R)rp.ambient, ambInv = (R)1 - ambient;
    const R floorLight = std::fmax((R)0, sun.y);
    const R sliceZ = (R)ph.gz * (R)0.5f;
    const V3<R> dinv{(R)1 / dir.x, (R)1 / dir.y, (R)1 / dir.z}, suninv{(R)1 / sun.x, (R)1 / sun.y, (R)1 / sun.z};
    const V3<R> smoke{(R)rp.smoke_color[0], (R)rp.smoke_color[1], (R)rp.smoke_color[2]};
    R dCurrent = 0, dSolid = (R)FLT_MAX, light;
    V3<R> color{0, 0, 0};
    R alpha = 0;
    int what = 0;
    if (rp.channel != DCG_RENDER_FLUID && (sliceZ - origin.z) * dir.z > (R)0) {
      const R d = (sliceZ - origin.z) / dir.z;
      const R px = origin.x + d * dir.x, py = origin.y + d * dir.y;
      if (px >= (R)0 && py >= (R)0 && px < (R)ph.gx && py < (R)ph.gy && d < dSolid) {
        dSolid = d;
        what = 3;
      }
    }
    if (rp.solids && ((R)0 - origin.y) * dir.y > (R)0) {
      const R d = ((R)0 - origin.y) / dir.y;
      if (d < dSolid) {
        dSolid = d;
        what = 2;
      }
    }
    if (rp.solids && ph.P->solids) {
      R s = (R)FLT_MAX, dScene = dCurrent;
      for (int i = 0; i < 100; i++) {
        s = sdf(origin + dir * dScene);
        if (s < (R)1e-1f || dScene >= dSolid) break;
        dScene += s;
      }
      if (s < (R)1e-1f && dScene < dSolid) {
        dSolid = dScene;
        what = 1;
      }
    }
    March<R> a;
    if (rp.channel == DCG_RENDER_FLUID) {
      R dNear, dFar;
      if (box_hit(dNear, dFar, origin, dinv)) {
        dCurrent = std::fmax(dCurrent, std::fmax(dNear, (R)10));
        V3<R> pos = origin + dir * dCurrent;
        const R dMax = std::fmin(dFar, dSolid);
        while (dCurrent < dMax && alpha <= (R)0.99f) {
          const V3<R> prev = pos;
          dCurrent = std::fmin(std::fmax(dCurrent * (R)1, dCurrent + (R)0.5f), dMax);
          pos = origin + dir * dCurrent;
          G.sample((prev + pos) * (R)0.5f, rp.precise != 0, a);
          if (a.density > (R)1e-6f) {
            const R sa = alpha_of(len3(pos - prev), a.density);
            light = 1;
            if (rp.shadows) light *= light_march((prev + pos) * (R)0.5f, sun, suninv);
            light = ambient + light * ambInv;
            mix3(smoke * light, sa, color, alpha);
          }
        }
      }
    }
    V3<R> pos = origin + dir * dSolid;
    const R bgAlpha = alpha_of(dSolid, (R)1e-6f);
    if (what == 1) {
      light = std::fmax((R)0, dot3(normal(pos), sun));
      if (rp.shadows) light *= light_march(pos, sun, suninv);
      light = ambient + light * ambInv;
      mix3(V3<R>{(R)rp.scene_color[0], (R)rp.scene_color[1], (R)rp.scene_color[2]} * light, (R)1 - bgAlpha, color,
           alpha);
    }
    if (what == 2) {
      pos.y = 0;
      light = floorLight;
      if (rp.shadows) light *= light_march(pos, sun, suninv);
      light = ambient + light * ambInv;
      light *= (R)1 + (R)0.1f * std::fmod(std::fabs(std::floor(pos.x / (R)ph.gx) + std::floor(pos.z / (R)ph.gx)), (R)2);
      mix3(V3<R>{(R)rp.floor_color[0], (R)rp.floor_color[1], (R)rp.floor_color[2]} * light, (R)1 - bgAlpha, color,
           alpha);
    }
    if (what == 3) {
      pos.z = sliceZ;
      G.sample(pos, rp.precise != 0, a);
      if (rp.channel == DCG_RENDER_DENSITY) mix3(V3<R>{a.density * (R)1e2f, 0, 0}, (R)1, color, alpha);
      if (rp.channel == DCG_RENDER_VELOCITY) {
        const R v = G.vel_len(a) * (R)1e-1f;
        mix3(V3<R>{v - (R)2, v - (R)1, v}, (R)1, color, alpha);
      }
      if (rp.channel == DCG_RENDER_RESOLUTION) {
        const R c = (R)((a.ix / 4 + a.iy / 4) % 2);
        mix3(V3<R>{c, c, c}, (R)1, color, alpha);
      }
      if (rp.channel == DCG_RENDER_FLUIDITY) {
        const R f = G.fluid(a);
        mix3(V3<R>{f, f, f}, (R)1, color, alpha);
      }
    }
    out[0] = color.x; out[1] = color.y; out[2] = color.z; out[3] = alpha;
  }
  void image(double *out) const {
    const R cx = (R)0.5f * (R)rp.width, cy = (R)0.5f * (R)rp.height;
    const R s = (R)rp.fov / std::fmax(cx, cy);
    const R step = (R)1 / (R)rp.aa_samples;
    const V3<R> origin = V3<R>{(R)rp.eye[0], (R)rp.eye[1], (R)rp.eye[2]} * ph.rdx;
    const V3<R> sun{(R)rp.sun_dir[0], (R)rp.sun_dir[1], (R)rp.sun_dir[2]};
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < rp.height; y++)
      for (int x = 0; x < rp.width; x++) {
        R acc[4] = {0, 0, 0, 0};
        for (R dx = 0; dx < (R)1; dx += step)
          for (R dy = 0; dy < (R)1; dy += step) {
            const V3<R> v = normalize3(V3<R>{((R)x + dx - cx) * s, ((R)y + dy - cy) * s, (R)1});
            const V3<R> dir{v.x, v.z * (R)rp.eye_dir[1] - v.y * (R)rp.eye_dir[2],
                            v.y * (R)rp.eye_dir[1] + v.z * (R)rp.eye_dir[2]};
            R c[4];
            march(origin, dir, sun, c);
            for (int k = 0; k < 4; k++) acc[k] += c[k];
          }
        for (int k = 0; k < 4; k++) out[((size_t)y * rp.width + x) * 4 + k] = (double)(acc[k] * (step * step));
      }
  }
};

// ======================================================================
//  Adaptive grid (DCGrid)
// ======================================================================
template <typename R> struct DC : Base {
  Physics<R> ph;
  int gx = 0, gy = 0, gz = 0, levels = 0, sparse = 0;
  int64_t B = 0;
  std::vector<int64_t> full, maxL, off, load, moveLimit;
  std::vector<int> bx, by, bz;
  std::vector<uint8_t> lvl, flags;
  std::vector<int64_t> parent, child, apron;
  std::vector<std::unordered_map<uint32_t, int64_t>> hash;
  int nq = 1;
  std::vector<R> q[3], v[3], w, p, pt, dv, tv[3], tq[3];
  std::vector<float> ss, bs;
  std::vector<int64_t> lastMoves, lastRefines, touched;
  int64_t lastMovedCount = 0, lastRefinedCount = 0;
  std::vector<R> emis;
  int set_emission(const double *src) override {
    const int n = P.emission_n;
    if (n <= 0) return fail(DCG_E_INVALID, "created with emission_n = 0");
    emis.assign(src, src + (size_t)n * n * n);
    return DCG_OK;
  }
  int set_heightmap(const float *h, int nx, int nz) override {
    const int rc = store_heightmap(h, nx, nz);
    if (rc) return rc;
    ph.set_heightmap(hmap, nx, nz);
    return reset();
  }

  R rdx() const { return ph.rdx; }

  // Level count and per-level budget split, fluid_simulation_dcgrid.cu:12-69.
  int create(const dcg_params &prm) {
    P = prm;
    mode = DCG_MODE_ADAPTIVE;
    gx = P.gx; gy = P.gy; gz = P.gz;
    if (gx <= 0 || gy <= 0 || gz <= 0) return fail(DCG_E_INVALID, "domain must be positive");
    if (P.dx <= 0.f) return fail(DCG_E_INVALID, "dx must be positive");
    if (P.jacobi_iters < 0 || (P.jacobi_iters & 1))
      return fail(DCG_E_INVALID, "jacobi_iters must be even and >= 0");
    if (P.n_scalars != 1 && P.n_scalars != 3) return fail(DCG_E_INVALID, "n_scalars must be 1 or 3");
    nq = P.n_scalars;
    rdx_f = 1.f / P.dx;
    ph.P = &P; ph.rdx = (R)rdx_f; ph.dt = (R)P.dt; ph.dx = (R)P.dx;
    ph.gx = gx; ph.gy = gy; ph.gz = gz;
    if (P.emission_n > 0) emis.assign((size_t)P.emission_n * P.emission_n * P.emission_n, (R)0);
    ph.em = &emis;
    const int minDim = std::min(gx, std::min(gy, gz));
    int cellSize = 2;
    levels = 1;
    while (gx % cellSize == 0 && gy % cellSize == 0 && gz % cellSize == 0 &&
           cellSize * BW <= minDim) {
      levels++;
      cellSize *= 2;
    }
    if (P.levels > 0) levels = P.levels;
    if (levels > 16) return fail(DCG_E_INVALID, "at most 16 levels");
    const int ext = BW << (levels - 1);
    if (gx % ext || gy % ext || gz % ext)
      return fail(DCG_E_INVALID, "domain must be a multiple of the coarsest block extent");
    full.assign(levels, 0); maxL.assign(levels, 0); off.assign(levels, 0);
    load.assign(levels, 0); moveLimit.assign(levels, 0);
    for (int l = 0, cs = 1; l < levels; l++, cs *= 2)
      full[l] = (int64_t)idiv_up(gx, cs * BW) * idiv_up(gy, cs * BW) * idiv_up(gz, cs * BW);
    B = P.max_blocks;
    if (B < full[levels - 1]) return fail(DCG_E_BUDGET, "too few blocks to fill the coarsest level");
    maxL[levels - 1] = full[levels - 1];
    int64_t left = B - maxL[levels - 1];
    for (int l = levels - 2; l >= 0; l--) {
      maxL[l] = std::min(left / (l + 1), full[l]);
      left -= maxL[l];
    }
    if (maxL[0] == 0) return fail(DCG_E_BUDGET, "too few blocks to reach the finest level");
    off[0] = 0;
    for (int l = 1; l < levels; l++) off[l] = off[l - 1] + maxL[l - 1];
    sparse = 0;
    for (int l = 0; l < levels; l++)
      if (maxL[l] < full[l]) sparse = l + 1;
    const size_t nc = (size_t)B * BV;
    bx.assign(B, 0); by.assign(B, 0); bz.assign(B, 0);
    lvl.assign(B, FREE); flags.assign(B, 0);
    parent.assign(B, NF); child.assign((size_t)B * 8, NF);
    apron.assign((size_t)B * AV, 0);
    hash.assign(levels, {});
    for (int k = 0; k < 3; k++) {
      q[k].assign(k < nq ? nc : 0, 0);
      tq[k].assign(k < nq ? nc : 0, 0);
      v[k].assign(nc, 0);
      tv[k].assign(nc, 0);
    }
    w.assign(nc, 0); p.assign(nc, 0); pt.assign(nc, 0); dv.assign(nc, 0);
    ss.assign((size_t)B * 8 + 1, 0.f);
    bs.assign(B, 0.f);
    return reset();
  }

  // ---------------- lookups ----------------
  // getBlockIndex (dcgrid_utils.cuh:169-199)
  int64_t get_block_index(int x, int y, int z, int level) const {
    if (level >= sparse) {
      const int extent = BW << level;
      const int64_t rx = idiv_up(gx, extent), ry = idiv_up(gy, extent), rz = idiv_up(gz, extent);
      const int px = x / BW, py = y / BW, pz = z / BW;
      if (px < 0 || py < 0 || pz < 0 || px >= rx || py >= ry || pz >= rz) return NF;
      return off[level] + ((int64_t)px * ry + py) * rz + pz;
    }
    auto it = hash[level].find(grid_hash(x, y, z));
    return it == hash[level].end() ? NF : it->second;
  }
  // getBlockIndexDeep (dcgrid_utils.cuh:201-233): the finest block at a level
  // >= `level` that contains the level-`level` cell (x, y, z). Updates level.
  int64_t deep(int x, int y, int z, int &level) const {
    if (level < sparse) {
      for (uint32_t key = grid_hash(x, y, z); level < sparse;
           level++, key >>= 3, x /= 2, y /= 2, z /= 2) {
        auto it = hash[level].find(key);
        if (it != hash[level].end()) return it->second;
      }
    }
    const int extent = BW << level;
    const int64_t rx = idiv_up(gx, extent), ry = idiv_up(gy, extent), rz = idiv_up(gz, extent);
    const int px = x / BW, py = y / BW, pz = z / BW;
    if (px >= rx || py >= ry || pz >= rz) return NF;
    return off[level] + ((int64_t)px * ry + py) * rz + pz;
  }
  void rebuild_hash() {
    for (auto &h : hash) h.clear();
    for (int64_t b = 0; b < B; b++)
      if (lvl[b] != FREE) hash[lvl[b]][grid_hash(bx[b], by[b], bz[b])] = b;
  }
  bool leaf(size_t cell) const { return child[cell >> 3] == NF; }

  // ---------------- reset / init ----------------
  // FluidSimulationDCGrid::reset (fluid_simulation_dcgrid.cu:212-261)
  int reset() override {
    std::fill(bx.begin(), bx.end(), 0); std::fill(by.begin(), by.end(), 0);
    std::fill(bz.begin(), bz.end(), 0);
    std::fill(lvl.begin(), lvl.end(), FREE);
    std::fill(flags.begin(), flags.end(), 0);
    std::fill(parent.begin(), parent.end(), NF);
    std::fill(child.begin(), child.end(), NF);
    std::fill(apron.begin(), apron.end(), 0);
    for (int k = 0; k < 3; k++) {
      std::fill(q[k].begin(), q[k].end(), (R)0);
      std::fill(v[k].begin(), v[k].end(), (R)0);
    }
    std::fill(w.begin(), w.end(), (R)0);
    std::fill(p.begin(), p.end(), (R)0);
    std::fill(pt.begin(), pt.end(), (R)0);
    std::fill(dv.begin(), dv.end(), (R)0);
    for (auto &h : hash) h.clear();
    for (int l = 0; l < levels; l++) {
      load[l] = (maxL[l] == full[l]) ? maxL[l] : 0;
      moveLimit[l] = 0;
    }
    steps = 0;
    return init();
  }

  // FluidSimulationDCGrid::init (cu:190-210)
  int init() {
    init_apron_indices();
    for (int l = sparse; l < levels; l++) activate_level(l);
    for (int i = 0; i < P.init_adapt_passes; i++) {
      int rc = adapt();
      if (rc) return rc;
    }
    if (P.src_enabled) {
      apply_sources_all();
      accumulate_q();
    }
    return DCG_OK;
  }

  // k_dcgrid_init_apron_indices (dcgrid_structure.cu:6-28)
  void init_apron_indices() {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      int64_t *a = &apron[(size_t)b * AV];
      for (int i = 0; i < AV; i++) a[i] = NF;
      for (int c = 0; c < BV; c++) {
        int x, y, z;
        local_xyz(c, x, y, z);
        a[AA * (1 + x) + AW * (1 + y) + (1 + z)] = b * BV + c;
      }
    }
  }

  // k_dcgrid_activate_level (dcgrid_structure.cu:104-178)
  void activate_level(int level) {
    const int scale = 1 << level, extent = BW << level;
    const int rx = idiv_up(gx, extent), ry = idiv_up(gy, extent), rz = idiv_up(gz, extent);
#pragma omp parallel for collapse(3) schedule(static)
    for (int tx = 0; tx < rx; tx++)
      for (int ty = 0; ty < ry; ty++)
        for (int tz = 0; tz < rz; tz++) {
          const int px = BW * tx, py = BW * ty, pz = BW * tz;
          if (px * scale >= gx || py * scale >= gy || pz * scale >= gz) continue;
          const int64_t b = get_block_index(px, py, pz, level);
          if (b == NF || b >= off[level] + maxL[level]) continue;
          bx[b] = px; by[b] = py; bz[b] = pz; lvl[b] = (uint8_t)level;
          if (level < levels - 1)
            parent[b] = 8 * get_block_index(px / 2, py / 2, pz / 2, level + 1) +
                        (px % (2 * BW)) + (py % (2 * BW)) / 2 + (pz % (2 * BW)) / 4;
          if (level - 1 >= sparse)
            for (int c = 0; c < 8; c++)
              child[8 * b + c] = get_block_index(2 * px + BW * ((c / 4) % 2),
                                                 2 * py + BW * ((c / 2) % 2),
                                                 2 * pz + BW * (c % 2), level - 1);
          int64_t *a = &apron[(size_t)b * AV];
          const int i0 = px > 0 ? 0 : 1, i1 = AW - ((px + BW) * scale >= gx ? 1 : 0);
          const int j0 = py > 0 ? 0 : 1, j1 = AW - ((py + BW) * scale >= gy ? 1 : 0);
          const int k0 = pz > 0 ? 0 : 1, k1 = AW - ((pz + BW) * scale >= gz ? 1 : 0);
          for (int i = i0; i < i1; i++)
            for (int j = j0; j < j1; j++)
              for (int k = k0; k < k1; k++) {
                const int64_t nb = get_block_index(px + i - 1, py + j - 1, pz + k - 1, level);
                a[AA * i + AW * j + k] =
                    nb * BV + local_of((i - 1 + BW) % BW, (j - 1 + BW) % BW, (k - 1 + BW) % BW);
              }
          for (int i = 0; i < AW; i++)
            for (int j = 0; j < AW; j++)
              for (int k = 0; k < AW; k++)
                if (a[AA * i + AW * j + k] == NF)
                  a[AA * i + AW * j + k] =
                      a[AA * clampi(i, 1, BW) + AW * clampi(j, 1, BW) + clampi(k, 1, BW)];
          for (int c = 0; c < BV; c++) {
            int x, y, z;
            local_xyz(c, x, y, z);
            const size_t cell = (size_t)b * BV + c;
            for (int k = 0; k < 3; k++) {
              if (k < nq) q[k][cell] = 0;
              v[k][cell] = 0;
            }
            w[cell] = ph.fluidity(px + x, py + y, pz + z, scale);
          }
        }
  }

  // ---------------- restriction ----------------
  // accumulate<T> + k_dcgrid_accumulate_* (dcgrid_structure.cu:188-222),
  // launched per level from fine to coarse (fluid_simulation_dcgrid.cu:496-515).
  // `scalars`: the fields are advected scalars (stored in the scalar format).
  void accumulate(std::vector<R> *const *fields, int nf, bool scalars = false) {
    for (int level = 0; level < levels - 1; level++) {
#pragma omp parallel for schedule(static)
      for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {
        if (lvl[b] != level || parent[b] == NF) continue;
        for (int s = 0; s < 8; s++) {
          const size_t pc = (size_t)parent[b] * 8 + s;
          for (int f = 0; f < nf; f++) {
            std::vector<R> &ch = *fields[f];
            R acc = 0;
            for (int i = 0; i < 8; i++) acc = acc + ch[(size_t)b * BV + 8 * s + i];
            ch[pc] = scalars ? store_q(acc * (R)0.125f, P.precision) : acc * (R)0.125f;
          }
        }
      }
    }
  }
  void accumulate_v() {
    std::vector<R> *f[3] = {&v[0], &v[1], &v[2]};
    accumulate(f, 3);
  }
  void accumulate_q() {
    std::vector<R> *f[3] = {&q[0], &q[1], &q[2]};
    accumulate(f, nq, true);
  }
  void accumulate_div() {
    std::vector<R> *f[1] = {&dv};
    accumulate(f, 1);
  }

  // ---------------- advection ----------------
  struct Sample {
    size_t idx[8];
    R wt[8];
    R wAcc;
    int x0, y0, z0, x1, y1, z1, scale;
  };
  // INIT_SAMPLE (dcgrid_fluid.cu:7-72)
  void sample(R pxw, R pyw, R pzw, Sample &s) const {
    int ix = clampi((int)std::floor(pxw), 0, gx - 1);
    int iy = clampi((int)std::floor(pyw), 0, gy - 1);
    int iz = clampi((int)std::floor(pzw), 0, gz - 1);
    int level = 0;
    const int64_t b = deep(ix, iy, iz, level);
    s.scale = 1 << level;
    const R scaleInv = (R)1 / (R)s.scale;
    const R x = pxw * scaleInv - (R)0.5f, y = pyw * scaleInv - (R)0.5f,
            z = pzw * scaleInv - (R)0.5f;
    const R xf = std::floor(x), yf = std::floor(y), zf = std::floor(z);
    const R dx = x - xf, dy = y - yf, dz = z - zf;
    s.x0 = (int)xf; s.y0 = (int)yf; s.z0 = (int)zf;
    s.x1 = s.x0 + 1; s.y1 = s.y0 + 1; s.z1 = s.z0 + 1;
    const int i = clampi(s.x1 - bx[b], 0, AW - 2);
    const int j = clampi(s.y1 - by[b], 0, AW - 2);
    const int k = clampi(s.z1 - bz[b], 0, AW - 2);
    const int64_t *a = &apron[(size_t)b * AV + AA * i + AW * j + k];
    s.idx[0] = a[0]; s.idx[1] = a[1]; s.idx[2] = a[AW]; s.idx[3] = a[AW + 1];
    s.idx[4] = a[AA]; s.idx[5] = a[AA + 1]; s.idx[6] = a[AA + AW]; s.idx[7] = a[AA + AW + 1];
    const R Dx = (R)1 - dx, Dy = (R)1 - dy, Dz = (R)1 - dz;
    s.wt[0] = w[s.idx[0]] * Dx * Dy * Dz;
    s.wt[1] = w[s.idx[1]] * Dx * Dy * dz;
    s.wt[2] = w[s.idx[2]] * Dx * dy * Dz;
    s.wt[3] = w[s.idx[3]] * Dx * dy * dz;
    s.wt[4] = w[s.idx[4]] * dx * Dy * Dz;
    s.wt[5] = w[s.idx[5]] * dx * Dy * dz;
    s.wt[6] = w[s.idx[6]] * dx * dy * Dz;
    s.wt[7] = w[s.idx[7]] * dx * dy * dz;
    s.wAcc = s.wt[0] + s.wt[1] + s.wt[2] + s.wt[3] + s.wt[4] + s.wt[5] + s.wt[6] + s.wt[7];
    const R wInv = (R)1 / s.wAcc;
    for (int c = 0; c < 8; c++) s.wt[c] = s.wt[c] * wInv;
  }
  void corner(const Sample &s, int c, int &x, int &y, int &z) const {
    x = (c & 4) ? s.x1 : s.x0;
    y = (c & 2) ? s.y1 : s.y0;
    z = (c & 1) ? s.z1 : s.z0;
  }
  // advectVelocity (dcgrid_fluid.cu:74-91)
  void sample_velocity(const Sample &s, R out[3]) const {
    out[0] = out[1] = out[2] = 0;
    if (s.wAcc < (R)1e-6f) return;
    for (int c = 0; c < 8; c++) {
      int x, y, z;
      corner(s, c, x, y, z);
      R vc[3] = {v[0][s.idx[c]], v[1][s.idx[c]], v[2][s.idx[c]]};
      ph.vel_bc(vc, x, y, z, s.scale);
      for (int d = 0; d < 3; d++) out[d] = (c == 0) ? vc[d] * s.wt[c] : out[d] + vc[d] * s.wt[c];
    }
  }
  // advectDensity (dcgrid_fluid.cu:93-110), for scalar k
  R sample_scalar(const Sample &s, int k) const {
    if (s.wAcc < (R)1e-6f) return 0;
    R out = 0;
    for (int c = 0; c < 8; c++) {
      int x, y, z;
      corner(s, c, x, y, z);
      const R qc = ph.q_bc(q[k][s.idx[c]], k, x, y, z, s.scale);
      out = (c == 0) ? qc * s.wt[c] : out + qc * s.wt[c];
    }
    return out;
  }
  void back_trace(int64_t b, int c, R out[3]) const {
    const R scale = (R)(1 << lvl[b]);
    const R alpha = ph.dt * ph.rdx;
    int x, y, z;
    local_xyz(c, x, y, z);
    const size_t cell = (size_t)b * BV + c;
    out[0] = ((R)(bx[b] + x) + (R)0.5f) * scale - v[0][cell] * alpha;
    out[1] = ((R)(by[b] + y) + (R)0.5f) * scale - v[1][cell] * alpha;
    out[2] = ((R)(bz[b] + z) + (R)0.5f) * scale - v[2][cell] * alpha;
  }

  // FluidSimulationDCGrid::advectVelocity (cu:263-268) with
  // k_dcgrid_advect_velocity (dcgrid_fluid.cu:112-127); buoyancy (extension)
  // is added to leaf cells from the scalars of the same cell.
  int advect_velocity() override {
    const bool buoy = P.buoy_alpha != 0.f || P.buoy_beta != 0.f;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        R out[3] = {0, 0, 0};
        if (leaf(cell)) {
          R pos[3];
          back_trace(b, c, pos);
          Sample s;
          sample(pos[0], pos[1], pos[2], s);
          sample_velocity(s, out);
          if (buoy) {
            R f = -(R)P.buoy_alpha * q[0][cell];
            if (nq > 1) f = f + (R)P.buoy_beta * (q[1][cell] - (R)P.t_ambient);
            out[1] = out[1] + ph.dt * f;
          }
        }
        for (int d = 0; d < 3; d++) tv[d][cell] = out[d];
      }
    }
    for (int d = 0; d < 3; d++) v[d].swap(tv[d]);
    accumulate_v();
    return DCG_OK;
  }

  void apply_sources_all() {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        int x, y, z;
        local_xyz(c, x, y, z);
        if (ph.in_source(bx[b] + x, by[b] + y, bz[b] + z, 1 << lvl[b]))
          for (int k = 0; k < nq; k++)
            q[k][cell] = store_q(ph.src_value_at(k, bx[b] + x, by[b] + y, bz[b] + z, lvl[b]), P.precision);
      }
    }
  }

  // FluidSimulationDCGrid::advectDensity (cu:313-318) with
  // k_dcgrid_advect_density (dcgrid_fluid.cu:129-144), for every scalar;
  // sphere sources (extension) overwrite leaf cells inside the source.
  int advect_scalars() override {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (leaf(cell)) {
          R pos[3];
          back_trace(b, c, pos);
          Sample s;
          sample(pos[0], pos[1], pos[2], s);
          for (int k = 0; k < nq; k++) tq[k][cell] = sample_scalar(s, k);
          int x, y, z;
          local_xyz(c, x, y, z);
          if (P.emission_n > 0)
            tq[0][cell] = tq[0][cell] + ph.dt * ph.emission_at(bx[b] + x, by[b] + y, bz[b] + z, 1 << lvl[b]);
          if (ph.in_source(bx[b] + x, by[b] + y, bz[b] + z, 1 << lvl[b]))
            for (int k = 0; k < nq; k++) tq[k][cell] = ph.src_value_at(k, bx[b] + x, by[b] + y, bz[b] + z, lvl[b]);
          for (int k = 0; k < nq; k++) tq[k][cell] = store_q(tq[k][cell], P.precision);
        } else {
          for (int k = 0; k < nq; k++) tq[k][cell] = 0;
        }
      }
    }
    for (int k = 0; k < nq; k++) q[k].swap(tq[k]);
    accumulate_q();
    return DCG_OK;
  }

  // ---------------- projection ----------------
  size_t apr(int64_t b, int i, int j, int k) const {
    return (size_t)apron[(size_t)b * AV + AA * i + AW * j + k];
  }
  // k_dcgrid_calc_divergence (dcgrid_fluid.cu:174-230)
  void calc_divergence() {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      const int scale = 1 << lvl[b];
      const R alpha = (R)0.5f * ph.rdx / (R)scale;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        p[cell] = 0; pt[cell] = 0; dv[cell] = 0;
      }
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int ax = lx + 1, ay = ly + 1, az = lz + 1;
        const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
        // neighbour velocity as staged in shared memory: own-block cells raw,
        // apron cells through velocityBndCond
        auto nv = [&](int di, int dj, int dk, int comp) -> R {
          const int i = ax + di, j = ay + dj, k = az + dk;
          const size_t n = apr(b, i, j, k);
          R vc[3] = {v[0][n], v[1][n], v[2][n]};
          if (i == 0 || i == AW - 1 || j == 0 || j == AW - 1 || k == 0 || k == AW - 1)
            ph.vel_bc(vc, x + di, y + dj, z + dk, scale);
          return vc[comp];
        };
        const R wl = w[apr(b, ax - 1, ay, az)], wr = w[apr(b, ax + 1, ay, az)];
        const R wd = w[apr(b, ax, ay - 1, az)], wu = w[apr(b, ax, ay + 1, az)];
        const R wb = w[apr(b, ax, ay, az - 1)], wf = w[apr(b, ax, ay, az + 1)];
        const R vlx = nv(-1, 0, 0, 0), vrx = nv(1, 0, 0, 0);
        const R vdy = nv(0, -1, 0, 1), vuy = nv(0, 1, 0, 1);
        const R vbz = nv(0, 0, -1, 2), vfz = nv(0, 0, 1, 2);
        dv[cell] = alpha * (wr * vrx - wl * vlx + wu * vuy - wd * vdy + wf * vfz - wb * vbz);
      }
    }
  }
  // k_dcgrid_jacobi / _inv (dcgrid_multigrid_solver.cu:5-41)
  void jacobi(int level, const std::vector<R> &src, std::vector<R> &dst) {
    const int s = 1 << level;
    const R alpha = (R)(s * s) * ph.dx * ph.dx;
#pragma omp parallel for schedule(static)
    for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {
      if (lvl[b] != level) continue;
      for (int c = 0; c < BV; c++) {
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int ax = lx + 1, ay = ly + 1, az = lz + 1;
        const size_t cell = (size_t)b * BV + c;
        const R pl = src[apr(b, ax - 1, ay, az)], pr = src[apr(b, ax + 1, ay, az)];
        const R pd = src[apr(b, ax, ay - 1, az)], pu = src[apr(b, ax, ay + 1, az)];
        const R pb = src[apr(b, ax, ay, az - 1)], pf = src[apr(b, ax, ay, az + 1)];
        dst[cell] = (pl + pr + pd + pu + pb + pf - alpha * dv[cell]) / (R)6;
      }
    }
  }
  // k_dcgrid_prolongate (dcgrid_multigrid_solver.cu:43-76)
  void prolongate(int level) {
#pragma omp parallel for schedule(static)
    for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {
      if (lvl[b] != level || parent[b] == NF) continue;
      const int64_t pb = parent[b] / 8;
      for (int c = 0; c < BV; c++) {
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
        const int px = (x / 2) % BW, py = (y / 2) % BW, pz = (z / 2) % BW;
        const int idx = AA * (1 + px) + AW * (1 + py) + (1 + pz);
        const int i = x % 2 ? AA : -AA, j = y % 2 ? AW : -AW, k = z % 2 ? 1 : -1;
        const int64_t *a = &apron[(size_t)pb * AV];
        const R p000 = p[a[idx]], p001 = p[a[idx + k]], p010 = p[a[idx + j]],
                p100 = p[a[idx + i]], p011 = p[a[idx + j + k]], p101 = p[a[idx + i + k]],
                p110 = p[a[idx + i + j]], p111 = p[a[idx + i + j + k]];
        p[(size_t)b * BV + c] = ((R)27 * p000 + (R)9 * (p001 + p010 + p100) +
                                 (R)3 * (p011 + p101 + p110) + p111) / (R)64;
      }
    }
  }
  // k_dcgrid_apply_pressure (dcgrid_fluid.cu:232-259)
  void apply_pressure() {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      const int scale = 1 << lvl[b];
      const R alpha = (R)0.5f * ph.rdx / (R)scale;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int ax = lx + 1, ay = ly + 1, az = lz + 1;
        const R pc = p[cell];
        const size_t L = apr(b, ax - 1, ay, az), Rr = apr(b, ax + 1, ay, az);
        const size_t D = apr(b, ax, ay - 1, az), U = apr(b, ax, ay + 1, az);
        const size_t Bk = apr(b, ax, ay, az - 1), F = apr(b, ax, ay, az + 1);
        v[0][cell] = v[0][cell] - alpha * (w[Rr] * (p[Rr] - pc) + w[L] * (pc - p[L]));
        v[1][cell] = v[1][cell] - alpha * (w[U] * (p[U] - pc) + w[D] * (pc - p[D]));
        v[2][cell] = v[2][cell] - alpha * (w[F] * (p[F] - pc) + w[Bk] * (pc - p[Bk]));
      }
    }
  }
  // FluidSimulationDCGrid::project (cu:270-294)
  // the cascade of FluidSimulationDCGrid::project (cu:274-290) on p / pt / dv
  void cascade() {
    const int pairs = P.jacobi_iters / 2;
    for (int i = 0; i < pairs; i++) {
      jacobi(levels - 1, p, pt);
      jacobi(levels - 1, pt, p);
    }
    for (int level = levels - 2; level >= 0; level--) {
      prolongate(level);
      for (int i = 0; i < pairs; i++) {
        jacobi(level, p, pt);
        jacobi(level, pt, p);
      }
    }
  }
  int project() override {
    calc_divergence();
    accumulate_div();
    cascade();
    if (P.defect_passes > 0) defect_correct();
    apply_pressure();
    accumulate_v();
    return DCG_OK;
  }
  // FP64 defect correction (extension): per pass the residual of every
  // allocated cell's Jacobi equation, r = div - (sum6 p - 6 p) / alpha, in
  // FP64 (stored in the field type), the cascade on r into e, p += e; a last
  // residual measures the result. dnorm[2k], dnorm[2k+1]: ||r||^2, ||div||^2.
  std::vector<R> e_, et_, rr_;
  std::vector<double> dnorm;
  void defect_correct() {
    const size_t nc = (size_t)B * BV;
    const int K = P.defect_passes;
    e_.assign(nc, 0); et_.assign(nc, 0); rr_.assign(nc, 0);
    dnorm.assign(2 * (K + 1), 0.0);
    for (int k = 0; k <= K; k++) {
      double r2 = 0, b2 = 0;
      for (int64_t b = 0; b < B; b++) {
        if (lvl[b] == FREE) continue;
        const int s = 1 << lvl[b];
        const R alpha = (R)(s * s) * ph.dx * ph.dx;
        for (int c = 0; c < BV; c++) {
          int lx, ly, lz;
          local_xyz(c, lx, ly, lz);
          const int ax = lx + 1, ay = ly + 1, az = lz + 1;
          const size_t cell = (size_t)b * BV + c;
          const double lap = (double)p[apr(b, ax - 1, ay, az)] + (double)p[apr(b, ax + 1, ay, az)] +
                             (double)p[apr(b, ax, ay - 1, az)] + (double)p[apr(b, ax, ay + 1, az)] +
                             (double)p[apr(b, ax, ay, az - 1)] + (double)p[apr(b, ax, ay, az + 1)] -
                             6.0 * (double)p[cell];
          const double r = (double)dv[cell] - lap / (double)alpha;
          rr_[cell] = (R)r;
          r2 += r * r;
          b2 += (double)dv[cell] * (double)dv[cell];
        }
      }
      dnorm[2 * k] = r2;
      dnorm[2 * k + 1] = b2;
      if (k == K) break;
      std::swap(p, e_);
      std::swap(pt, et_);
      std::swap(dv, rr_);
      std::fill(p.begin(), p.end(), (R)0);
      cascade();
      std::swap(p, e_);
      std::swap(pt, et_);
      std::swap(dv, rr_);
      for (int64_t b = 0; b < B; b++) {
        if (lvl[b] == FREE) continue;
        for (int c = 0; c < BV; c++) p[(size_t)b * BV + c] = p[(size_t)b * BV + c] + e_[(size_t)b * BV + c];
      }
    }
  }
  // FluidSimulationDCGrid::projectLocal (cu:296-311): 2x the pairs per level,
  // coarse to fine, no prolongation.
  int project_local() override {
    calc_divergence();
    accumulate_div();
    const int pairs = P.jacobi_iters;
    for (int level = levels - 1; level >= 0; level--)
      for (int i = 0; i < pairs; i++) {
        jacobi(level, p, pt);
        jacobi(level, pt, p);
      }
    apply_pressure();
    accumulate_v();
    return DCG_OK;
  }

  // ---------------- adaptation ----------------
  bool level_blocked(int level) const {
    return (level == 0 && load[0] == full[0]) ||
           (level > 0 && load[level - 1] == full[level - 1]);
  }
  // Field criterion (extension): max over the subblock's cells of
  // max(|curl v| / vort_threshold, |grad rho| / grad_threshold), with the
  // central differences of k_dcgrid_calc_vorticity (dcgrid_fluid.cu:146-172).
  R cell_field_score(int64_t b, int c) const {
    int lx, ly, lz;
    local_xyz(c, lx, ly, lz);
    const int ax = lx + 1, ay = ly + 1, az = lz + 1;
    const int scale = 1 << lvl[b];
    const R alpha = (R)0.5f * ph.rdx / (R)scale;
    const size_t L = apr(b, ax - 1, ay, az), Rr = apr(b, ax + 1, ay, az);
    const size_t D = apr(b, ax, ay - 1, az), U = apr(b, ax, ay + 1, az);
    const size_t Bk = apr(b, ax, ay, az - 1), F = apr(b, ax, ay, az + 1);
    const R wl = w[L], wr = w[Rr], wd = w[D], wu = w[U], wb = w[Bk], wf = w[F];
    const R ox = alpha * ((wu * v[2][U] - wd * v[2][D]) - (wf * v[1][F] - wb * v[1][Bk]));
    const R oy = alpha * ((wf * v[0][F] - wb * v[0][Bk]) - (wr * v[2][Rr] - wl * v[2][L]));
    const R oz = alpha * ((wr * v[1][Rr] - wl * v[1][L]) - (wu * v[0][U] - wd * v[0][D]));
    const R gxr = alpha * (q[0][Rr] - q[0][L]);
    const R gyr = alpha * (q[0][U] - q[0][D]);
    const R gzr = alpha * (q[0][F] - q[0][Bk]);
    const R om = std::sqrt(ox * ox + oy * oy + oz * oz);
    const R gr = std::sqrt(gxr * gxr + gyr * gyr + gzr * gzr);
    return std::max(om / (R)P.vort_threshold, gr / (R)P.grad_threshold);
  }
  // k_dcgrid_calc_subblock_scores (dcgrid_adaptation.cu:10-40)
  void calc_subblock_scores() {
#pragma omp parallel for schedule(static)
    for (int64_t sb = 0; sb < B * 8; sb++) {
      const int64_t b = sb / 8;
      const uint8_t level = lvl[b];
      if (child[sb] != NF || level == FREE || level_blocked(level)) {
        ss[sb] = -FLT_MAX;
        continue;
      }
      if (P.refine_criterion == DCG_REFINE_GEOMETRIC) {
        const float sc = (float)(1 << level);
        const float px = sc * ((float)bx[b] + 2.f * (float)((sb >> 2) & 1) + 1.f);
        const float py = sc * ((float)by[b] + 2.f * (float)((sb >> 1) & 1) + 1.f);
        const float pz = sc * ((float)bz[b] + 2.f * (float)(sb & 1) + 1.f);
        const float ddx = px - .5f * (float)gx, ddy = py - .45f * (float)gy,
                    ddz = pz - .5f * (float)gz;
        const float d = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
        ss[sb] = d < .2f * (float)gx ? 0.f : (float)gx / d;
      } else {
        R m = 0;
        for (int i = 0; i < 8; i++) m = std::max(m, cell_field_score(b, (int)(sb % 8) * 8 + i));
        ss[sb] = (float)m;
      }
    }
    ss[(size_t)B * 8] = 0.f;  // the slot past the end read by the compat block score
  }
  // k_dcgrid_accumulate_subblock_scores (dcgrid_adaptation.cu:42-63). With
  // ref_compat the ninth summand s[8] (the next block's first subblock) is kept.
  void accumulate_subblock_scores() {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      bs[b] = -FLT_MAX;
      const uint8_t level = lvl[b];
      if (level == FREE || level_blocked(level)) continue;
      const float *s = &ss[(size_t)b * 8];
      if (s[0] > 0.f && s[1] > 0.f && s[2] > 0.f && s[3] > 0.f && s[4] > 0.f &&
          s[5] > 0.f && s[6] > 0.f && s[7] > 0.f) {
        float sum = s[0] + s[1] + s[2] + s[3] + s[4] + s[5] + s[6] + s[7];
        if (P.ref_compat) sum = sum + s[8];
        bs[b] = .125f * sum;
      }
    }
  }
  // FluidSimulationDCGrid::moveBlocks (cu:348-437). Orders: blocks ascending
  // by score with negative scores last, subblocks descending; equal keys are
  // ordered by index (one of the orders std::sort/nth_element may produce).
  void select_moves(std::vector<std::pair<int64_t, int64_t>> &pairs) {
    calc_subblock_scores();
    accumulate_subblock_scores();
    std::fill(flags.begin(), flags.end(), 0);
    pairs.clear();
    for (int level = 0; level < levels - 1; level++) {
      const int64_t d0 = maxL[level], d1 = 8 * maxL[level + 1];
      int64_t l = std::min({d0, d1, load[level], full[level] - load[level]});
      if (moveLimit[level] > 0) l = std::min(l, moveLimit[level]);
      if (l == 0) continue;
      std::vector<int64_t> mc(d0), dc(d1);
      std::iota(mc.begin(), mc.end(), off[level]);
      std::iota(dc.begin(), dc.end(), 8 * off[level + 1]);
      auto blockLess = [this](int64_t a, int64_t b) {
        const bool na = bs[a] < 0.f, nb = bs[b] < 0.f;
        if (na != nb) return nb;  // negatives last
        if (!na && bs[a] != bs[b]) return bs[a] < bs[b];
        return a < b;
      };
      auto subLess = [this](int64_t a, int64_t b) {
        if (ss[a] != ss[b]) return ss[a] > ss[b];
        return a < b;
      };
      const int64_t nsort_b = std::min(d0, l + 1), nsort_s = std::min(d1, l + 1);
      std::partial_sort(mc.begin(), mc.begin() + nsort_b, mc.end(), blockLess);
      std::partial_sort(dc.begin(), dc.begin() + nsort_s, dc.end(), subLess);
      int64_t matches = 0;
      while (matches < l && bs[mc[matches]] >= 0.f && ss[dc[matches]] >= 0.f &&
             bs[mc[matches]] < ss[dc[matches]]) {
        matches++;
        if (P.ref_compat) {
          // the reference protects the block of the *next* candidate (cu:415-417)
          if (matches < d1) bs[dc[matches] / 8] = -FLT_MAX;
        } else {
          bs[dc[matches - 1] / 8] = -FLT_MAX;
        }
      }
      moveLimit[level] = (int64_t)(size_t)((float)matches * 1.2f);
      for (int64_t m = 0; m < matches; m++) pairs.push_back({mc[m], dc[m]});
    }
  }
  // k_dcgrid_move_blocks (dcgrid_adaptation.cu:65-90). Coarser levels are
  // applied first so that a block moved into a block that moves in the same
  // pass takes its parent's new position.
  void apply_moves(const std::vector<std::pair<int64_t, int64_t>> &pairs) {
    for (int level = levels - 2; level >= 0; level--)
      for (const auto &pr : pairs) {
        const int64_t b = pr.first, dest = pr.second;
        if (lvl[b] != level) continue;
        const int64_t prev = parent[b];
        if (prev != NF) child[prev] = NF;
        child[dest] = b;
        parent[b] = dest;
        const int64_t pb = dest / 8;
        bx[b] = 2 * bx[pb] + BW * (int)((dest / 4) % 2);
        by[b] = 2 * by[pb] + BW * (int)((dest / 2) % 2);
        bz[b] = 2 * bz[pb] + BW * (int)(dest % 2);
        flags[b] |= MOVED;
        flags[pb] |= REFINED;
      }
  }
  // FluidSimulationDCGrid::refineSubblocks (cu:439-483). ref_compat keeps the
  // refineLimit largest subblock *indices* (the reference's nth_element with
  // std::greater over indices); otherwise the highest scores.
  void select_refines(std::vector<int64_t> &subs) {
    calc_subblock_scores();
    subs.clear();
    for (int level = 1; level < levels; level++) {
      const uint64_t a = (uint64_t)(maxL[level - 1] - load[level - 1]);
      const uint64_t b = (uint64_t)(8 * load[level]) - (uint64_t)load[level - 1];
      const int64_t limit = (int64_t)std::min(a, b);
      if (limit == 0) continue;
      std::vector<int64_t> cand;
      for (int64_t i = 8 * off[level]; i < 8 * off[level] + 8 * maxL[level]; i++)
        if (ss[i] > P.refine_threshold) cand.push_back(i);
      if ((int64_t)cand.size() > limit) {
        if (P.ref_compat) {
          cand.erase(cand.begin(), cand.end() - limit);
        } else {
          std::stable_sort(cand.begin(), cand.end(),
                           [this](int64_t x, int64_t y) { return ss[x] > ss[y]; });
          cand.resize(limit);
          std::sort(cand.begin(), cand.end());
        }
      }
      subs.insert(subs.end(), cand.begin(), cand.end());
    }
  }
  // k_dcgrid_refine_subblocks + insertBlock (dcgrid_adaptation.cu:145-178,
  // dcgrid_utils.cuh:99-140). New blocks are allocated in list order.
  int64_t refine_one(int64_t sb) {
    const int64_t pb = sb / 8;
    const int level = lvl[pb];
    const int cx = 2 * bx[pb] + BW * (int)((sb / 4) % 2);
    const int cy = 2 * by[pb] + BW * (int)((sb / 2) % 2);
    const int cz = 2 * bz[pb] + BW * (int)(sb % 2);
    const int cl = level - 1;
    const uint32_t key = grid_hash(cx, cy, cz);
    int64_t cb;
    auto it = hash[cl].find(key);
    if (it != hash[cl].end()) {
      cb = it->second;
    } else {
      if (load[cl] >= maxL[cl]) return NF;
      cb = off[cl] + load[cl]++;
      hash[cl][key] = cb;
      bx[cb] = cx; by[cb] = cy; bz[cb] = cz; lvl[cb] = (uint8_t)cl;
    }
    parent[cb] = sb;
    child[sb] = cb;
    flags[pb] |= REFINED;
    flags[cb] |= MOVED;
    return cb;
  }
  // k_dcgrid_refresh_apron_indices (dcgrid_structure.cu:30-92). Out-of-domain
  // entries of moved blocks are set with SPREAD(clamp(i,1,4)) as in the
  // reference (local coordinate i mod 4) when ref_compat is on. The
  // reference's refresh goes at most one level deeper for an entry whose
  // block was refined: when a block moves into a place and one of its
  // subblocks is refined in the same adaptation, a neighbour keeps pointing at
  // the moved (coarser) block until a later refresh. ref_compat keeps that;
  // without it every entry is the finest block's (a fresh lookup).
  void refresh_apron() {
    if (!P.ref_compat) {
      rebuild_apron_fresh();
      return;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      const int level = lvl[b];
      for (int ai = 0; ai < AV; ai++) {
        const int i = (ai / AA) % AW, j = (ai / AW) % AW, k = ai % AW;
        if (i % (AW - 1) != 0 && j % (AW - 1) != 0 && k % (AW - 1) != 0) continue;
        int64_t &entry = apron[(size_t)b * AV + ai];
        int64_t nb = NF;
        if (flags[b] & MOVED) {
          const int nx = bx[b] + i - 1, ny = by[b] + j - 1, nz = bz[b] + k - 1;
          const int scale = 1 << level;
          if (nx < 0 || ny < 0 || nz < 0 || nx * scale >= gx || ny * scale >= gy ||
              nz * scale >= gz) {
            entry = b * BV + out_local(i, j, k, level);
            continue;
          }
          int nl = level;
          nb = deep(nx, ny, nz, nl);
        } else {
          const int64_t prev = entry / BV;
          const uint8_t cf = flags[prev];
          if (cf & MOVED) {
            int nl = level;
            nb = deep(bx[b] + i - 1, by[b] + j - 1, bz[b] + k - 1, nl);
          } else if ((cf & REFINED) && lvl[prev] > level) {
            nb = child[entry / 8];
          }
        }
        if (nb == NF) continue;
        const int s = 1 << (lvl[nb] - level);
        const int x = (bx[b] + i - 1) / s - bx[nb];
        const int y = (by[b] + j - 1) / s - by[nb];
        const int z = (bz[b] + k - 1) / s - bz[nb];
        entry = nb * BV + local_of(x, y, z);
      }
    }
  }
  int out_local(int i, int j, int k, int level) const {
    if (P.ref_compat && level < sparse)
      return spread(clampi(i, 1, BW), 2) + spread(clampi(j, 1, BW), 1) + spread(clampi(k, 1, BW), 0);
    return local_of(clampi(i, 1, BW) - 1, clampi(j, 1, BW) - 1, clampi(k, 1, BW) - 1);
  }
  // The apron entry a fresh deep lookup gives (used to check the incremental
  // refresh and to rebuild aprons of a replaced topology).
  int64_t fresh_entry(int64_t b, int i, int j, int k) const {
    const int level = lvl[b];
    if (i >= 1 && i <= BW && j >= 1 && j <= BW && k >= 1 && k <= BW)
      return b * BV + local_of(i - 1, j - 1, k - 1);
    const int nx = bx[b] + i - 1, ny = by[b] + j - 1, nz = bz[b] + k - 1;
    const int scale = 1 << level;
    if (nx < 0 || ny < 0 || nz < 0 || nx * scale >= gx || ny * scale >= gy || nz * scale >= gz)
      return b * BV + out_local(i, j, k, level);
    int nl = level;
    const int64_t nb = level >= sparse ? get_block_index(nx, ny, nz, level) : deep(nx, ny, nz, nl);
    if (nb == NF) return NF;
    const int s = 1 << (lvl[nb] - level);
    return nb * BV + local_of(nx / s - bx[nb], ny / s - by[nb], nz / s - bz[nb]);
  }
  // k_dcgrid_propagate_values (dcgrid_adaptation.cu:92-143)
  void propagate(int level) {
#pragma omp parallel for schedule(static)
    for (size_t t = 0; t < touched.size(); t++) {
      const int64_t b = touched[t];
      if (b == NF || lvl[b] != level || parent[b] == NF) continue;
      const int64_t pb = parent[b] / 8;
      const int scale = 1 << level;
      const int64_t *a = &apron[(size_t)pb * AV];
      for (int c = 0; c < BV; c++) {
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
        const int px = (x / 2) % BW, py = (y / 2) % BW, pz = (z / 2) % BW;
        const int idx = AA * (1 + px) + AW * (1 + py) + (1 + pz);
        const int i = x % 2 ? AA : -AA, j = y % 2 ? AW : -AW, k = z % 2 ? 1 : -1;
        const size_t i000 = a[idx], i001 = a[idx + k], i010 = a[idx + j], i100 = a[idx + i],
                     i011 = a[idx + j + k], i101 = a[idx + i + k], i110 = a[idx + i + j],
                     i111 = a[idx + i + j + k];
        const size_t cell = (size_t)b * BV + c;
        auto tri = [&](const std::vector<R> &f) {
          return (R)(27.f / 64.f) * f[i000] + (R)(9.f / 64.f) * (f[i001] + f[i010] + f[i100]) +
                 (R)(3.f / 64.f) * (f[i011] + f[i101] + f[i110]) + (R)(1.f / 64.f) * f[i111];
        };
        for (int kq = 0; kq < nq; kq++) q[kq][cell] = store_q(tri(q[kq]), P.precision);
        for (int d = 0; d < 3; d++) v[d][cell] = tri(v[d]);
        w[cell] = ph.fluidity(x, y, z, scale);
      }
    }
  }
  // FluidSimulationDCGrid::adaptTopology (cu:320-346)
  int adapt() override {
    std::vector<std::pair<int64_t, int64_t>> pairs;
    select_moves(pairs);
    std::vector<int64_t> subs;
    return apply_adapt(pairs, subs, false);
  }
  int apply_adapt(const std::vector<std::pair<int64_t, int64_t>> &pairs,
                  std::vector<int64_t> &subs, bool replay_refines,
                  const std::vector<int64_t> *replay_blocks = nullptr) {
    if (replay_refines) std::fill(flags.begin(), flags.end(), 0);
    apply_moves(pairs);
    touched.clear();
    lastMoves.clear();
    lastRefines.clear();
    for (const auto &pr : pairs) {
      touched.push_back(pr.first);
      lastMoves.push_back(pr.first);
      lastMoves.push_back(pr.second);
    }
    if (!pairs.empty()) rebuild_hash();
    if (!replay_refines) select_refines(subs);
    for (size_t r = 0; r < subs.size(); r++) {
      const int64_t cb = refine_one(subs[r]);
      if (replay_blocks && cb != (*replay_blocks)[r]) return fail(DCG_E_INVALID, "replayed refinement allocated a different block");
      touched.push_back(cb);
      lastRefines.push_back(subs[r]);
      lastRefines.push_back(cb);
    }
    lastMovedCount = (int64_t)pairs.size();
    lastRefinedCount = (int64_t)subs.size();
    if (!touched.empty()) {
      refresh_apron();
      for (int level = levels - 2; level >= 0; level--) propagate(level);
    }
    return DCG_OK;
  }
  int replay(const int64_t *moves, int64_t nm, const int64_t *refines, int64_t nr) {
    std::vector<std::pair<int64_t, int64_t>> pairs;
    for (int64_t i = 0; i < nm; i++) pairs.push_back({moves[2 * i], moves[2 * i + 1]});
    std::vector<int64_t> subs, blocks;
    for (int64_t i = 0; i < nr; i++) {
      subs.push_back(refines[2 * i]);
      blocks.push_back(refines[2 * i + 1]);
    }
    // block scores / move limits follow the same bookkeeping as a selection
    return apply_adapt(pairs, subs, true, &blocks);
  }

  int add_noise(uint64_t seed, float amp) override {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int c = 0; c < BV; c++) {
        int x, y, z;
        local_xyz(c, x, y, z);
        const size_t cell = (size_t)b * BV + c;
        for (int d = 0; d < 3; d++)
          v[d][cell] = v[d][cell] + (R)(amp * noise_unit(seed, bx[b] + x, by[b] + y, bz[b] + z, lvl[b], d));
      }
    }
    return DCG_OK;
  }

  // ---------------- access ----------------
  std::vector<R> *field_ptr(int f) {
    switch (f) {
      case DCG_FIELD_DENSITY: return &q[0];
      case DCG_FIELD_VEL_X: return &v[0];
      case DCG_FIELD_VEL_Y: return &v[1];
      case DCG_FIELD_VEL_Z: return &v[2];
      case DCG_FIELD_FLUIDITY: return &w;
      case DCG_FIELD_PRESSURE: return &p;
      case DCG_FIELD_PRESSURE_TMP: return &pt;
      case DCG_FIELD_DIVERGENCE: return &dv;
      case DCG_FIELD_TEMPERATURE: return nq > 1 ? &q[1] : nullptr;
      case DCG_FIELD_VAPOR: return nq > 2 ? &q[2] : nullptr;
    }
    return nullptr;
  }
  int get_field(int f, double *dst) override {
    auto *fp = field_ptr(f);
    if (!fp) return fail(DCG_E_NOT_FOUND, "no such field");
    for (size_t i = 0; i < fp->size(); i++) dst[i] = (double)(*fp)[i];
    return DCG_OK;
  }
  int set_field(int f, const double *src) override {
    auto *fp = field_ptr(f);
    if (!fp) return fail(DCG_E_NOT_FOUND, "no such field");
    const bool narrow = P.precision != DCG_PRECISION_FP32 &&
                        (f == DCG_FIELD_DENSITY || f == DCG_FIELD_TEMPERATURE || f == DCG_FIELD_VAPOR);
    for (size_t i = 0; i < fp->size(); i++)
      (*fp)[i] = narrow ? store_q((R)(float)src[i], P.precision) : (R)src[i];
    return DCG_OK;
  }
  int get_dense(int f, double *dst) override {
    auto *fp = field_ptr(f);
    if (!fp) return fail(DCG_E_NOT_FOUND, "no such field");
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          int level = 0;
          const int64_t b = deep(x, y, z, level);
          const int lx = (x >> level) - bx[b], ly = (y >> level) - by[b], lz = (z >> level) - bz[b];
          dst[((size_t)z * gy + y) * gx + x] = (double)(*fp)[(size_t)b * BV + local_of(lx, ly, lz)];
        }
    return DCG_OK;
  }
  // ---------------- adjoint of the density path ----------------
  // Transpose of the step that produced the current state, with its flow and
  // topology held fixed: restriction^T, (advection + emission)^T with source
  // cells cut, then the transpose of the propagation into touched blocks.
  // Serial loops: the scatters need no atomics.
  void adjoint_step(const double *lam_in, double *lam_out, double *lam_em) {
    const size_t nc = (size_t)B * BV;
    std::vector<double> lam(lam_in, lam_in + nc);
    for (int level = levels - 2; level >= 0; level--)
      for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {
        if (lvl[b] != level || parent[b] == NF) continue;
        for (int s = 0; s < 8; s++) {
          const size_t pc = (size_t)parent[b] * 8 + s;
          const double lp = lam[pc] * 0.125;
          for (int i = 0; i < 8; i++) lam[(size_t)b * BV + 8 * s + i] += lp;
          lam[pc] = 0;
        }
      }
    std::fill(lam_out, lam_out + nc, 0.0);
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell) || lam[cell] == 0) continue;
        int x, y, z;
        local_xyz(c, x, y, z);
        const int scale = 1 << lvl[b];
        if (ph.in_source(bx[b] + x, by[b] + y, bz[b] + z, scale)) continue;
        if (P.emission_n > 0 && lam_em)
          ph.emission_adjoint(bx[b] + x, by[b] + y, bz[b] + z, scale, (double)ph.dt * lam[cell], lam_em);
        R pos[3];
        back_trace(b, c, pos);
        Sample s;
        sample(pos[0], pos[1], pos[2], s);
        if (s.wAcc < (R)1e-6f) continue;
        for (int k = 0; k < 8; k++) {
          int cx, cy, cz;
          corner(s, k, cx, cy, cz);
          if (ph.q_passes(cx, cy, cz, s.scale)) lam_out[s.idx[k]] += lam[cell] * (double)s.wt[k];
        }
      }
    }
    for (int level = 0; level <= levels - 2; level++)
      for (size_t t = 0; t < touched.size(); t++) {
        const int64_t b = touched[t];
        if (b == NF || lvl[b] != level || parent[b] == NF) continue;
        const int64_t pb = parent[b] / 8;
        const int64_t *a = &apron[(size_t)pb * AV];
        for (int c = 0; c < BV; c++) {
          int lx, ly, lz;
          local_xyz(c, lx, ly, lz);
          const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
          const int px = (x / 2) % BW, py = (y / 2) % BW, pz = (z / 2) % BW;
          const int idx = AA * (1 + px) + AW * (1 + py) + (1 + pz);
          const int i = x % 2 ? AA : -AA, j = y % 2 ? AW : -AW, k = z % 2 ? 1 : -1;
          const size_t cell = (size_t)b * BV + c;
          const double l = lam_out[cell];
          lam_out[cell] = 0;
          lam_out[a[idx]] += 27.0 / 64.0 * l;
          lam_out[a[idx + k]] += 9.0 / 64.0 * l;
          lam_out[a[idx + j]] += 9.0 / 64.0 * l;
          lam_out[a[idx + i]] += 9.0 / 64.0 * l;
          lam_out[a[idx + j + k]] += 3.0 / 64.0 * l;
          lam_out[a[idx + i + k]] += 3.0 / 64.0 * l;
          lam_out[a[idx + i + j]] += 3.0 / 64.0 * l;
          lam_out[a[idx + i + j + k]] += 1.0 / 64.0 * l;
        }
      }
  }
  // ---------------- full adjoint of one step ----------------
  // The whole state (velocity and every scalar): buoyancy, the pressure
  // projection (every Jacobi sweep and prolongation of the cascade
  // transposed, in reverse order) and the dependence of the semi-Lagrangian
  // sample positions on the velocity, with the block topology recorded. The
  // simulation holds the state before the step; the step runs (replaying the
  // given adaptation decisions when `moves` is not null) and its stages'
  // transposes are applied in reverse order in FP64. Afterwards the
  // simulation holds the state after the step. lam_in / lam_out: (3 + nq)
  // planes of B*64: v_x, v_y, v_z, the scalars.
  using VD = std::vector<double>;
  void adj_restrict(VD &lam) const {
    for (int level = levels - 2; level >= 0; level--)
      for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {
        if (lvl[b] != level || parent[b] == NF) continue;
        for (int s = 0; s < 8; s++) {
          const size_t pc = (size_t)parent[b] * 8 + s;
          const double lp = lam[pc] * 0.125;
          for (int i = 0; i < 8; i++) lam[(size_t)b * BV + 8 * s + i] += lp;
          lam[pc] = 0;
        }
      }
  }
  void adj_propagate(VD &lam) const {
    for (int level = 0; level <= levels - 2; level++)
      for (size_t t = 0; t < touched.size(); t++) {
        const int64_t b = touched[t];
        if (b == NF || lvl[b] != level || parent[b] == NF) continue;
        const int64_t pb = parent[b] / 8;
        const int64_t *a = &apron[(size_t)pb * AV];
        for (int c = 0; c < BV; c++) {
          int lx, ly, lz;
          local_xyz(c, lx, ly, lz);
          const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
          const int px = (x / 2) % BW, py = (y / 2) % BW, pz = (z / 2) % BW;
          const int idx = AA * (1 + px) + AW * (1 + py) + (1 + pz);
          const int i = x % 2 ? AA : -AA, j = y % 2 ? AW : -AW, k = z % 2 ? 1 : -1;
          const size_t cell = (size_t)b * BV + c;
          const double l = lam[cell];
          lam[cell] = 0;
          lam[a[idx]] += 27.0 / 64.0 * l;
          lam[a[idx + k]] += 9.0 / 64.0 * l;
          lam[a[idx + j]] += 9.0 / 64.0 * l;
          lam[a[idx + i]] += 9.0 / 64.0 * l;
          lam[a[idx + j + k]] += 3.0 / 64.0 * l;
          lam[a[idx + i + k]] += 3.0 / 64.0 * l;
          lam[a[idx + i + j]] += 3.0 / 64.0 * l;
          lam[a[idx + i + j + k]] += 1.0 / 64.0 * l;
        }
      }
  }
  // d(w_c * trilinear_c) / d(fractional coordinate a) of a sample
  void sample_derivs(const Sample &s, R pxw, R pyw, R pzw, double dW[3][8], double G[3]) const {
    const R scaleInv = (R)1 / (R)s.scale;
    const R x = pxw * scaleInv - (R)0.5f, y = pyw * scaleInv - (R)0.5f, z = pzw * scaleInv - (R)0.5f;
    const double dx = (double)(x - std::floor(x)), dy = (double)(y - std::floor(y)), dz = (double)(z - std::floor(z));
    G[0] = G[1] = G[2] = 0;
    for (int c = 0; c < 8; c++) {
      const double wc = (double)w[s.idx[c]];
      const double X = (c & 4) ? dx : 1 - dx, Y = (c & 2) ? dy : 1 - dy, Z = (c & 1) ? dz : 1 - dz;
      const double sx = (c & 4) ? 1 : -1, sy = (c & 2) ? 1 : -1, sz = (c & 1) ? 1 : -1;
      dW[0][c] = wc * sx * Y * Z;
      dW[1][c] = wc * X * sy * Z;
      dW[2][c] = wc * X * Y * sz;
      for (int a = 0; a < 3; a++) G[a] += dW[a][c];
    }
  }
  // velocity advection + buoyancy transpose, on the state before the step
  void adj_velocity(VD *lv, VD *out_v, VD *out_q) const {
    for (int d = 0; d < 3; d++) adj_restrict(lv[d]);
    const bool buoy = P.buoy_alpha != 0.f || P.buoy_beta != 0.f;
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        const double l[3] = {lv[0][cell], lv[1][cell], lv[2][cell]};
        if (l[0] == 0 && l[1] == 0 && l[2] == 0) continue;
        if (buoy) {
          out_q[0][cell] += -(double)ph.dt * (double)P.buoy_alpha * l[1];
          if (nq > 1) out_q[1][cell] += (double)ph.dt * (double)P.buoy_beta * l[1];
        }
        R pos[3];
        back_trace(b, c, pos);
        Sample s;
        sample(pos[0], pos[1], pos[2], s);
        if (s.wAcc < (R)1e-6f) continue;
        double dW[3][8], G[3];
        sample_derivs(s, pos[0], pos[1], pos[2], dW, G);
        double gsum[3] = {0, 0, 0};
        for (int k = 0; k < 8; k++) {
          int x, y, z;
          corner(s, k, x, y, z);
          R vc[3] = {v[0][s.idx[k]], v[1][s.idx[k]], v[2][s.idx[k]]};
          ph.vel_bc(vc, x, y, z, s.scale);
          const bool pass = ph.q_passes(x, y, z, s.scale);
          for (int comp = 0; comp < 3; comp++) {
            if (pass) out_v[comp][s.idx[k]] += l[comp] * (double)s.wt[k];
            for (int a = 0; a < 3; a++) gsum[a] += l[comp] * dW[a][k] * (double)vc[comp];
          }
        }
        double out[3] = {0, 0, 0};
        for (int k = 0; k < 8; k++)
          for (int comp = 0; comp < 3; comp++) {
            int x, y, z;
            corner(s, k, x, y, z);
            R vc[3] = {v[0][s.idx[k]], v[1][s.idx[k]], v[2][s.idx[k]]};
            ph.vel_bc(vc, x, y, z, s.scale);
            out[comp] += (double)s.wt[k] * (double)vc[comp];
          }
        for (int a = 0; a < 3; a++)
          for (int comp = 0; comp < 3; comp++) gsum[a] -= l[comp] * out[comp] * G[a];
        const double f = -(double)(ph.dt * ph.rdx) / (double)s.scale / (double)s.wAcc;
        for (int a = 0; a < 3; a++) out_v[a][cell] += f * gsum[a];
      }
    }
  }
  int adjoint_step_full(const double *lam_in, double *lam_out, double *lam_em, const int64_t *moves, int64_t nm,
                        const int64_t *refines, int64_t nr) {
    if (P.defect_passes) return fail(DCG_E_INVALID, "the full adjoint does not transpose the defect correction");
    const size_t nc = (size_t)B * BV;
    DC before = *this;
    before.ph.P = &before.P;
    before.ph.em = &before.emis;
    advect_velocity();
    int rc = moves ? replay(moves, nm, refines, nr) : adapt();
    if (rc) return rc;
    std::vector<R> q0p[3];
    for (int k = 0; k < nq; k++) q0p[k] = q[k];
    project();
    advect_scalars();
    steps++;
    // phase A on the state after the step
    VD lv[3], lq[3], out_v[3], out_q[3];
    for (int d = 0; d < 3; d++) {
      lv[d].assign(lam_in + d * nc, lam_in + (d + 1) * nc);
      out_v[d].assign(nc, 0.0);
    }
    for (int k = 0; k < nq; k++) {
      lq[k].assign(lam_in + (3 + k) * nc, lam_in + (4 + k) * nc);
      out_q[k].assign(nc, 0.0);
      adj_restrict(lq[k]);
    }
    for (int64_t b = 0; b < B; b++) {  // scalar advection (+ emission, sources cut)
      if (lvl[b] == FREE) continue;
      const int scale0 = 1 << lvl[b];
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        bool any = false;
        for (int k = 0; k < nq; k++) any |= lq[k][cell] != 0;
        if (!any) continue;
        int x, y, z;
        local_xyz(c, x, y, z);
        if (ph.in_source(bx[b] + x, by[b] + y, bz[b] + z, scale0)) continue;
        if (P.emission_n > 0 && lam_em && lq[0][cell] != 0)
          ph.emission_adjoint(bx[b] + x, by[b] + y, bz[b] + z, scale0, (double)ph.dt * lq[0][cell], lam_em);
        R pos[3];
        back_trace(b, c, pos);
        Sample s;
        sample(pos[0], pos[1], pos[2], s);
        if (s.wAcc < (R)1e-6f) continue;
        double dW[3][8], G[3];
        sample_derivs(s, pos[0], pos[1], pos[2], dW, G);
        double gsum[3] = {0, 0, 0};
        for (int k = 0; k < nq; k++) {
          const double l = lq[k][cell];
          if (l == 0) continue;
          double out = 0, H[3] = {0, 0, 0};
          for (int cc = 0; cc < 8; cc++) {
            int cx, cy, cz;
            corner(s, cc, cx, cy, cz);
            const double val = (double)ph.q_bc(q0p[k][s.idx[cc]], k, cx, cy, cz, s.scale);
            out += (double)s.wt[cc] * val;
            for (int a = 0; a < 3; a++) H[a] += dW[a][cc] * val;
            if (ph.q_passes(cx, cy, cz, s.scale)) out_q[k][s.idx[cc]] += l * (double)s.wt[cc];
          }
          for (int a = 0; a < 3; a++) gsum[a] += l * (H[a] - out * G[a]) / (double)s.wAcc;
        }
        const double f = -(double)(ph.dt * ph.rdx) / (double)s.scale;
        for (int a = 0; a < 3; a++) lv[a][cell] += f * gsum[a];
      }
    }
    for (int d = 0; d < 3; d++) adj_restrict(lv[d]);
    VD lp[2] = {VD(nc, 0.0), VD(nc, 0.0)}, ld(nc, 0.0);
    for (int64_t b = 0; b < B; b++) {  // pressure gradient
      if (lvl[b] == FREE) continue;
      const double alpha = (double)((R)0.5f * ph.rdx / (R)(1 << lvl[b]));
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int ax = lx + 1, ay = ly + 1, az = lz + 1;
        for (int a = 0; a < 3; a++) {
          const double l = lv[a][cell];
          if (l == 0) continue;
          const size_t L = apr(b, ax - (a == 0), ay - (a == 1), az - (a == 2));
          const size_t Rr = apr(b, ax + (a == 0), ay + (a == 1), az + (a == 2));
          const double wL = (double)w[L], wR = (double)w[Rr];
          lp[0][Rr] += -alpha * wR * l;
          lp[0][cell] += -alpha * (wL - wR) * l;
          lp[0][L] += alpha * wL * l;
        }
      }
    }
    const int sweeps = P.jacobi_iters;
    for (int level = 0; level < levels; level++) {  // the cascade, transposed
      const int s = 1 << level;
      const double alpha = (double)((R)(s * s) * ph.dx * ph.dx);
      for (int it = sweeps - 1; it >= 0; it--) {
        VD &ldst = lp[(it & 1) ? 0 : 1], &lsrc = lp[(it & 1) ? 1 : 0];
#pragma omp parallel for schedule(static)
        for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {
          if (lvl[b] != level) continue;
          for (int c = 0; c < BV; c++) {
            const size_t cell = (size_t)b * BV + c;
            const double l = ldst[cell];
            if (l == 0) continue;
            ldst[cell] = 0;
            int lx, ly, lz;
            local_xyz(c, lx, ly, lz);
            const int ax = lx + 1, ay = ly + 1, az = lz + 1;
            const size_t nb[6] = {apr(b, ax - 1, ay, az), apr(b, ax + 1, ay, az), apr(b, ax, ay - 1, az),
                                  apr(b, ax, ay + 1, az), apr(b, ax, ay, az - 1), apr(b, ax, ay, az + 1)};
            for (int n = 0; n < 6; n++) {
#pragma omp atomic
              lsrc[nb[n]] += l / 6.0;
            }
            ld[cell] += -alpha * l / 6.0;
          }
        }
      }
      if (level == levels - 1) break;
      for (int64_t b = off[level]; b < off[level] + maxL[level]; b++) {  // prolongation
        if (lvl[b] != level || parent[b] == NF) continue;
        const int64_t pb = parent[b] / 8;
        const int64_t *a = &apron[(size_t)pb * AV];
        for (int c = 0; c < BV; c++) {
          const size_t cell = (size_t)b * BV + c;
          const double l = lp[0][cell];
          lp[0][cell] = 0;
          if (l == 0) continue;
          int lx, ly, lz;
          local_xyz(c, lx, ly, lz);
          const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
          const int px = (x / 2) % BW, py = (y / 2) % BW, pz = (z / 2) % BW;
          const int idx = AA * (1 + px) + AW * (1 + py) + (1 + pz);
          const int i = x % 2 ? AA : -AA, j = y % 2 ? AW : -AW, k = z % 2 ? 1 : -1;
          lp[0][a[idx]] += 27.0 / 64.0 * l;
          lp[0][a[idx + k]] += 9.0 / 64.0 * l;
          lp[0][a[idx + j]] += 9.0 / 64.0 * l;
          lp[0][a[idx + i]] += 9.0 / 64.0 * l;
          lp[0][a[idx + j + k]] += 3.0 / 64.0 * l;
          lp[0][a[idx + i + k]] += 3.0 / 64.0 * l;
          lp[0][a[idx + i + j]] += 3.0 / 64.0 * l;
          lp[0][a[idx + i + j + k]] += 1.0 / 64.0 * l;
        }
      }
    }
    adj_restrict(ld);
    for (int64_t b = 0; b < B; b++) {  // divergence
      if (lvl[b] == FREE) continue;
      const int scale = 1 << lvl[b];
      const double alpha = (double)((R)0.5f * ph.rdx / (R)scale);
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell) || ld[cell] == 0) continue;
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int ax = lx + 1, ay = ly + 1, az = lz + 1;
        const int x = bx[b] + lx, y = by[b] + ly, z = bz[b] + lz;
        for (int a = 0; a < 3; a++)
          for (int sg = -1; sg <= 1; sg += 2) {
            const int da = a == 0 ? sg : 0, db = a == 1 ? sg : 0, dc = a == 2 ? sg : 0;
            if (!ph.q_passes(x + da, y + db, z + dc, scale)) continue;
            const size_t n = apr(b, ax + da, ay + db, az + dc);
            lv[a][n] += (double)sg * alpha * (double)w[n] * ld[cell];
          }
      }
    }
    for (int d = 0; d < 3; d++) adj_propagate(lv[d]);
    for (int k = 0; k < nq; k++) adj_propagate(out_q[k]);
    // phase B on the state before the step
    before.adj_velocity(lv, out_v, out_q);
    for (int d = 0; d < 3; d++) std::copy(out_v[d].begin(), out_v[d].end(), lam_out + d * nc);
    for (int k = 0; k < nq; k++) std::copy(out_q[k].begin(), out_q[k].end(), lam_out + (3 + k) * nc);
    return DCG_OK;
  }
  // transpose of get_dense: lam_cells[leaf covering (x,y,z)] += lam_dense[x,y,z]
  void adjoint_dense(const double *lam_dense, double *lam_cells) const {
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          int level = 0;
          const int64_t b = deep(x, y, z, level);
          const int lx = (x >> level) - bx[b], ly = (y >> level) - by[b], lz = (z >> level) - bz[b];
          lam_cells[(size_t)b * BV + local_of(lx, ly, lz)] += lam_dense[((size_t)z * gy + y) * gx + x];
        }
  }
  // ---------------- renderer samplers (dcgrid_rendering.cu:6-56) ----------------
  struct Sampler {
    const DC &d;
    void sample(V3<R> p, bool precise, March<R> &a) const {
      a.ix = clampi((int)std::floor(p.x), 0, d.gx - 1);
      a.iy = clampi((int)std::floor(p.y), 0, d.gy - 1);
      a.iz = clampi((int)std::floor(p.z), 0, d.gz - 1);
      int level = 0;
      const int64_t b = d.deep(a.ix, a.iy, a.iz, level);
      if (!precise) {
        const int sh = d.P.ref_compat ? 0 : level;  // the reference uses the finest coordinates mod 4
        const size_t c = (size_t)b * BV + local_of((a.ix >> sh) & 3, (a.iy >> sh) & 3, (a.iz >> sh) & 3);
        for (int k = 0; k < 8; k++) a.idx[k] = c;
        a.fx = a.fy = a.fz = 0;
        a.density = d.q[0][c];
        return;
      }
      const R si = (R)1 / (R)(1 << level);
      const R x = p.x * si - (R)0.5f, y = p.y * si - (R)0.5f, z = p.z * si - (R)0.5f;
      const R xf = std::floor(x), yf = std::floor(y), zf = std::floor(z);
      a.fx = x - xf; a.fy = y - yf; a.fz = z - zf;
      const int i = (int)xf + 1 - d.bx[b], j = (int)yf + 1 - d.by[b], k = (int)zf + 1 - d.bz[b];
      const int64_t *ap = &d.apron[(size_t)b * AV + AA * i + AW * j + k];
      a.idx[0] = ap[0]; a.idx[1] = ap[1]; a.idx[2] = ap[AW]; a.idx[3] = ap[AW + 1];
      a.idx[4] = ap[AA]; a.idx[5] = ap[AA + 1]; a.idx[6] = ap[AA + AW]; a.idx[7] = ap[AA + AW + 1];
      a.density = interp(a, [&](size_t c) { return d.q[0][c]; });
    }
    R vel_len(const March<R> &a) const {
      const R vx = interp(a, [&](size_t c) { return d.v[0][c]; });
      const R vy = interp(a, [&](size_t c) { return d.v[1][c]; });
      const R vz = interp(a, [&](size_t c) { return d.v[2][c]; });
      return std::sqrt(vx * vx + vy * vy + vz * vz);
    }
    R fluid(const March<R> &a) const { return interp(a, [&](size_t c) { return d.w[c]; }); }
  };
  int render(const dcg_render_params &rp, double *out) const override {
    Sampler S{*this};
    Marcher<R, Sampler>{S, ph, rp}.image(out);
    return DCG_OK;
  }

  // this simulation takes another one's whole state (same parameters)
  void copy_state_from(const DC &o) {
    *this = o;
    ph.P = &P;
    ph.em = &emis;
  }

  void info(dcg_info *i) const override {
    std::memset(i, 0, sizeof(*i));
    i->mode = DCG_MODE_ADAPTIVE;
    i->levels = levels;
    i->sparse_levels = sparse;
    i->n_scalars = nq;
    i->max_blocks = B;
    i->num_cells = B * BV;
    for (int l = 0; l < levels; l++) {
      i->full_blocks[l] = full[l];
      i->budget[l] = maxL[l];
      i->offset[l] = off[l];
    }
  }
  // k_dcgrid_debug_stats (dcgrid_structure.cu:224-251) in the precision R
  // (its FP32 arithmetic for R = float) + leaf counts and mass; FP64 sums.
  int stats(dcg_stats *st) override {
    std::memset(st, 0, sizeof(*st));
    double res = 0, mass = 0;
    std::vector<int64_t> leafc(levels, 0);
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      const int scale = 1 << lvl[b];
      const R alpha = (R)rdx_f * (R)rdx_f / (R)(scale * scale);
      for (int c = 0; c < BV; c++) {
        const size_t cell = (size_t)b * BV + c;
        if (!leaf(cell)) continue;
        leafc[lvl[b]]++;
        int lx, ly, lz;
        local_xyz(c, lx, ly, lz);
        const int ax = lx + 1, ay = ly + 1, az = lz + 1;
        const R lap = p[apr(b, ax - 1, ay, az)] + p[apr(b, ax + 1, ay, az)] + p[apr(b, ax, ay - 1, az)] +
                      p[apr(b, ax, ay + 1, az)] + p[apr(b, ax, ay, az - 1)] + p[apr(b, ax, ay, az + 1)] -
                      (R)6 * p[cell];
        const R r = dv[cell] - lap * alpha;
        res += (double)((R)scale * std::fabs(r));
        mass += (double)(q[0][cell] * w[cell] * (R)(scale * scale * scale));
      }
    }
    for (int l = 0; l < levels; l++) {
      st->load[l] = load[l];
      st->leaf_cells[l] = leafc[l];
      st->active_cells += leafc[l];
    }
    st->moved_blocks = lastMovedCount;
    st->refined_subblocks = lastRefinedCount;
    st->steps = steps;
    st->residual = res;
    st->mass = mass;
    if (P.defect_passes > 0 && !dnorm.empty()) {
      const int K = P.defect_passes;
      auto rel = [](double r2, double b2) { return b2 > 0 ? std::sqrt(r2 / b2) : 0.0; };
      st->defect_rel_residual[0] = rel(dnorm[0], dnorm[1]);
      st->defect_rel_residual[1] = rel(dnorm[2 * K], dnorm[2 * K + 1]);
    }
    return DCG_OK;
  }
  int64_t apron_mismatches() const {
    int64_t n = 0;
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int ai = 0; ai < AV; ai++)
        if (apron[(size_t)b * AV + ai] != fresh_entry(b, ai / AA, (ai / AW) % AW, ai % AW)) n++;
    }
    return n;
  }
  void rebuild_apron_fresh() {
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < B; b++) {
      if (lvl[b] == FREE) continue;
      for (int ai = 0; ai < AV; ai++)
        apron[(size_t)b * AV + ai] = fresh_entry(b, ai / AA, (ai / AW) % AW, ai % AW);
    }
  }
};

// ======================================================================
//  Uniform grid (FluidSimulationUniform)
// ======================================================================
template <typename R> struct UG : Base {
  Physics<R> ph;
  int gx = 0, gy = 0, gz = 0, levels = 0;
  size_t nc = 0, nmip = 0;
  int nq = 1;
  std::vector<R> emis;
  int set_emission(const double *src) override {
    const int n = P.emission_n;
    if (n <= 0) return fail(DCG_E_INVALID, "created with emission_n = 0");
    emis.assign(src, src + (size_t)n * n * n);
    return DCG_OK;
  }
  int set_heightmap(const float *h, int nx, int nz) override {
    const int rc = store_heightmap(h, nx, nz);
    if (rc) return rc;
    ph.set_heightmap(hmap, nx, nz);
    return reset();
  }
  std::vector<R> q[3], v[3], w, p, pt, dv, tv[3], tq[3];

  // mipmapCells / mipmapIdx (src/utils/grid_math.cuh:24-52)
  size_t mip_cells() const {
    size_t n = 0;
    for (size_t s = 1; gx % s == 0 && gy % s == 0 && gz % s == 0 && s <= (size_t)(1 << (levels - 1)); s *= 2)
      n += ((size_t)gx * gy * gz) / (s * s * s);
    return n;
  }
  size_t mip_idx(int x, int y, int z, int scale) const {
    size_t o = 0;
    for (size_t s = 1; s < (size_t)scale; s *= 2) o += ((size_t)gx * gy * gz) / (s * s * s);
    return o + ((size_t)z * (gy / scale) + y) * (gx / scale) + x;
  }
  size_t idx3(int x, int y, int z) const { return ((size_t)z * gy + y) * gx + x; }

  int create(const dcg_params &prm) {
    P = prm;
    mode = DCG_MODE_UNIFORM;
    gx = P.gx; gy = P.gy; gz = P.gz;
    if (gx <= 0 || gy <= 0 || gz <= 0) return fail(DCG_E_INVALID, "domain must be positive");
    if (P.dx <= 0.f) return fail(DCG_E_INVALID, "dx must be positive");
    if (P.n_scalars != 1 && P.n_scalars != 3) return fail(DCG_E_INVALID, "n_scalars must be 1 or 3");
    nq = P.n_scalars;
    rdx_f = 1.f / P.dx;
    ph.P = &P; ph.rdx = (R)rdx_f; ph.dt = (R)P.dt; ph.dx = (R)P.dx;
    ph.gx = gx; ph.gy = gy; ph.gz = gz;
    if (P.emission_n > 0) emis.assign((size_t)P.emission_n * P.emission_n * P.emission_n, (R)0);
    ph.em = &emis;
    // FluidSimulationUniform ctor (fluid_simulation_uniform.cu:6-18)
    const int minDim = std::min(gx, std::min(gy, gz));
    int cellSize = 2;
    levels = 1;
    while (gx % cellSize == 0 && gy % cellSize == 0 && gz % cellSize == 0 && cellSize * 4 <= minDim) {
      levels++;
      cellSize *= 2;
    }
    if (P.levels > 0) levels = P.levels;
    const int top = 1 << (levels - 1);
    if (gx % top || gy % top || gz % top)
      return fail(DCG_E_INVALID, "domain must be divisible by 2^(levels-1)");
    nc = (size_t)gx * gy * gz;
    nmip = mip_cells();
    for (int k = 0; k < 3; k++) {
      q[k].assign(k < nq ? nc : 0, 0);
      tq[k].assign(k < nq ? nc : 0, 0);
      v[k].assign(nc, 0);
      tv[k].assign(nc, 0);
    }
    w.assign(nmip, 0); p.assign(nmip, 0); pt.assign(nmip, 0); dv.assign(nmip, 0);
    return reset();
  }
  // reset / init / adaptTopology (fluid_simulation_uniform.cu:76-92,143-147)
  int reset() override {
    for (int k = 0; k < 3; k++) {
      std::fill(q[k].begin(), q[k].end(), (R)0);
      std::fill(v[k].begin(), v[k].end(), (R)0);
    }
    std::fill(p.begin(), p.end(), (R)0);
    std::fill(w.begin(), w.end(), (R)0);
    std::fill(pt.begin(), pt.end(), (R)0);
    std::fill(dv.begin(), dv.end(), (R)0);
    steps = 0;
    adapt();
    if (P.src_enabled) apply_sources_all();
    return DCG_OK;
  }
  // k_uniform_set_solidity_ratio (uniformgrid_structure.cu:23-31)
  int adapt() override {
    for (int l = 0; l < levels; l++) {
      const int s = 1 << l;
#pragma omp parallel for collapse(2) schedule(static)
      for (int z = 0; z < gz / s; z++)
        for (int y = 0; y < gy / s; y++)
          for (int x = 0; x < gx / s; x++) w[mip_idx(x, y, z, s)] = ph.fluidity(x, y, z, s);
    }
    return DCG_OK;
  }
  void apply_sources_all() {
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++)
          if (ph.in_source(x, y, z, 1))
            for (int k = 0; k < nq; k++) q[k][idx3(x, y, z)] = ph.src_value_at(k, x, y, z, 0);
  }
  struct Sample {
    size_t idx[8];
    R wt[8];
    R wAcc;
    int x0, y0, z0, x1, y1, z1;
  };
  // INIT_SAMPLE (uniformgrid_fluid.cu:7-48)
  void sample(R px, R py, R pz, Sample &s) const {
    const R x = px - (R)0.5f, y = py - (R)0.5f, z = pz - (R)0.5f;
    const R xf = std::floor(x), yf = std::floor(y), zf = std::floor(z);
    s.x0 = (int)xf; s.y0 = (int)yf; s.z0 = (int)zf;
    s.x1 = s.x0 + 1; s.y1 = s.y0 + 1; s.z1 = s.z0 + 1;
    const int x0c = clampi(s.x0, 0, gx - 1), y0c = clampi(s.y0, 0, gy - 1), z0c = clampi(s.z0, 0, gz - 1);
    const int x1c = clampi(s.x1, 0, gx - 1), y1c = clampi(s.y1, 0, gy - 1), z1c = clampi(s.z1, 0, gz - 1);
    s.idx[0] = idx3(x0c, y0c, z0c); s.idx[1] = idx3(x0c, y0c, z1c);
    s.idx[2] = idx3(x0c, y1c, z0c); s.idx[3] = idx3(x0c, y1c, z1c);
    s.idx[4] = idx3(x1c, y0c, z0c); s.idx[5] = idx3(x1c, y0c, z1c);
    s.idx[6] = idx3(x1c, y1c, z0c); s.idx[7] = idx3(x1c, y1c, z1c);
    const R dx = x - xf, dy = y - yf, dz = z - zf;
    const R Dx = (R)1 - dx, Dy = (R)1 - dy, Dz = (R)1 - dz;
    s.wt[0] = w[s.idx[0]] * Dx * Dy * Dz;
    s.wt[1] = w[s.idx[1]] * Dx * Dy * dz;
    s.wt[2] = w[s.idx[2]] * Dx * dy * Dz;
    s.wt[3] = w[s.idx[3]] * Dx * dy * dz;
    s.wt[4] = w[s.idx[4]] * dx * Dy * Dz;
    s.wt[5] = w[s.idx[5]] * dx * Dy * dz;
    s.wt[6] = w[s.idx[6]] * dx * dy * Dz;
    s.wt[7] = w[s.idx[7]] * dx * dy * dz;
    s.wAcc = s.wt[0] + s.wt[1] + s.wt[2] + s.wt[3] + s.wt[4] + s.wt[5] + s.wt[6] + s.wt[7];
    const R wInv = (R)1 / s.wAcc;
    for (int c = 0; c < 8; c++) s.wt[c] = s.wt[c] * wInv;
  }
  void corner(const Sample &s, int c, int &x, int &y, int &z) const {
    x = (c & 4) ? s.x1 : s.x0;
    y = (c & 2) ? s.y1 : s.y0;
    z = (c & 1) ? s.z1 : s.z0;
  }
  void back_trace(int x, int y, int z, R out[3]) const {
    const size_t i = idx3(x, y, z);
    // make_float3(x, y, z) + .5f - velocity * dt * rdx (uniformgrid_fluid.cu:88-96)
    out[0] = ((R)x + (R)0.5f) - v[0][i] * ph.dt * ph.rdx;
    out[1] = ((R)y + (R)0.5f) - v[1][i] * ph.dt * ph.rdx;
    out[2] = ((R)z + (R)0.5f) - v[2][i] * ph.dt * ph.rdx;
  }
  // k_uniform_advect_velocity (uniformgrid_fluid.cu:88-96) + buoyancy (extension)
  int advect_velocity() override {
    const bool buoy = P.buoy_alpha != 0.f || P.buoy_beta != 0.f;
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          R pos[3];
          back_trace(x, y, z, pos);
          Sample s;
          sample(pos[0], pos[1], pos[2], s);
          R out[3] = {0, 0, 0};
          if (!(s.wAcc < (R)1e-6f))
            for (int c = 0; c < 8; c++) {
              int cx, cy, cz;
              corner(s, c, cx, cy, cz);
              R vc[3] = {v[0][s.idx[c]], v[1][s.idx[c]], v[2][s.idx[c]]};
              ph.vel_bc(vc, cx, cy, cz, 1);
              for (int d = 0; d < 3; d++) out[d] = (c == 0) ? vc[d] * s.wt[c] : out[d] + vc[d] * s.wt[c];
            }
          const size_t i = idx3(x, y, z);
          if (buoy) {
            R f = -(R)P.buoy_alpha * q[0][i];
            if (nq > 1) f = f + (R)P.buoy_beta * (q[1][i] - (R)P.t_ambient);
            out[1] = out[1] + ph.dt * f;
          }
          for (int d = 0; d < 3; d++) tv[d][i] = out[d];
        }
    for (int d = 0; d < 3; d++) v[d].swap(tv[d]);
    return DCG_OK;
  }
  // k_uniform_advect_density (uniformgrid_fluid.cu:98-105) for each scalar + sources
  int advect_scalars() override {
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          R pos[3];
          back_trace(x, y, z, pos);
          Sample s;
          sample(pos[0], pos[1], pos[2], s);
          const size_t i = idx3(x, y, z);
          for (int k = 0; k < nq; k++) {
            R out = 0;
            if (!(s.wAcc < (R)1e-6f))
              for (int c = 0; c < 8; c++) {
                int cx, cy, cz;
                corner(s, c, cx, cy, cz);
                const R qc = ph.q_bc(q[k][s.idx[c]], k, cx, cy, cz, 1);
                out = (c == 0) ? qc * s.wt[c] : out + qc * s.wt[c];
              }
            if (k == 0 && P.emission_n > 0) out = out + ph.dt * ph.emission_at(x, y, z, 1);
            tq[k][i] = out;
          }
          if (ph.in_source(x, y, z, 1))
            for (int k = 0; k < nq; k++) tq[k][i] = ph.src_value_at(k, x, y, z, 0);
        }
    for (int k = 0; k < nq; k++) q[k].swap(tq[k]);
    return DCG_OK;
  }
  // k_uniform_calc_divergence (uniformgrid_fluid.cu:107-132)
  void calc_divergence() {
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          const size_t i = idx3(x, y, z);
          const size_t il = x > 0 ? i - 1 : i, ir = x < gx - 1 ? i + 1 : i;
          const size_t id = y > 0 ? i - gx : i, iu = y < gy - 1 ? i + gx : i;
          const size_t ib = z > 0 ? i - (size_t)gx * gy : i, iff = z < gz - 1 ? i + (size_t)gx * gy : i;
          p[i] = 0; pt[i] = 0; dv[i] = 0;
          auto nv = [&](size_t n, int cx, int cy, int cz, int comp) {
            R vc[3] = {v[0][n], v[1][n], v[2][n]};
            ph.vel_bc(vc, cx, cy, cz, 1);
            return vc[comp];
          };
          const R vl = nv(il, x - 1, y, z, 0), vr = nv(ir, x + 1, y, z, 0);
          const R vd = nv(id, x, y - 1, z, 1), vu = nv(iu, x, y + 1, z, 1);
          const R vb = nv(ib, x, y, z - 1, 2), vf = nv(iff, x, y, z + 1, 2);
          dv[i] = (R)0.5f * ph.rdx *
                  (w[ir] * vr - w[il] * vl + w[iu] * vu - w[id] * vd + w[iff] * vf - w[ib] * vb);
        }
  }
  // k_uniform_restrict (uniformgrid_fluid.cu:134-160)
  void restrict_level(int l) {
    const int scale = 1 << l, cs = scale / 2;
    const int wc = gx / cs, hc = gy / cs;
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz / scale; z++)
      for (int y = 0; y < gy / scale; y++)
        for (int x = 0; x < gx / scale; x++) {
          const size_t i = mip_idx(x, y, z, scale);
          const size_t i000 = mip_idx(2 * x, 2 * y, 2 * z, cs);
          const size_t i001 = i000 + 1, i010 = i000 + wc, i011 = i010 + 1;
          const size_t i100 = i000 + (size_t)wc * hc, i101 = i100 + 1, i110 = i100 + wc, i111 = i110 + 1;
          p[i] = 0; pt[i] = 0;
          dv[i] = (R)0.125f * (dv[i000] + dv[i001] + dv[i010] + dv[i011] + dv[i100] + dv[i101] +
                               dv[i110] + dv[i111]);
        }
  }
  // calcPressure (uniformgrid_fluid.cu:162-192)
  void jacobi(int l, const std::vector<R> &src, std::vector<R> &dst) {
    const int scale = 1 << l;
    const R alpha = ph.dx * ph.dx * (R)scale * (R)scale;
    const int ww = gx / scale, hh = gy / scale, dd = gz / scale;
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < dd; z++)
      for (int y = 0; y < hh; y++)
        for (int x = 0; x < ww; x++) {
          const size_t i = mip_idx(x, y, z, scale);
          const size_t il = x > 0 ? i - 1 : i, ir = x < ww - 1 ? i + 1 : i;
          const size_t id = y > 0 ? i - ww : i, iu = y < hh - 1 ? i + ww : i;
          const size_t ib = z > 0 ? i - (size_t)ww * hh : i, iff = z < dd - 1 ? i + (size_t)ww * hh : i;
          dst[i] = (src[il] + src[ir] + src[id] + src[iu] + src[ib] + src[iff] - alpha * dv[i]) / (R)6;
        }
  }
  // k_uniform_prolongate (uniformgrid_fluid.cu:206-237)
  void prolongate(int l) {
    const int scale = 1 << l;
    const int ww = gx / scale, hh = gy / scale, dd = gz / scale;
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < dd; z++)
      for (int y = 0; y < hh; y++)
        for (int x = 0; x < ww; x++) {
          const size_t i = mip_idx(x, y, z, scale);
          const size_t i000 = mip_idx(x / 2, y / 2, z / 2, 2 * scale);
          const int sx = (x == 0 || x == ww - 1) ? 0 : 2 * (x % 2) - 1;
          const int sy = (y == 0 || y == hh - 1) ? 0 : 2 * (y % 2) - 1;
          const int sz = (z == 0 || z == dd - 1) ? 0 : 2 * (z % 2) - 1;
          const size_t i001 = i000 + sx;
          const size_t i010 = i000 + (int64_t)sy * ww / 2;
          const size_t i011 = i010 + sx;
          const size_t i100 = i000 + (int64_t)sz * (ww / 2) * (hh / 2);
          const size_t i101 = i100 + sx;
          const size_t i110 = i100 + (int64_t)sy * (ww / 2);
          const size_t i111 = i110 + sx;
          p[i] = ((R)27 * p[i000] + (R)9 * (p[i001] + p[i010] + p[i100]) +
                  (R)3 * (p[i011] + p[i101] + p[i110]) + p[i111]) / (R)64;
        }
  }
  // k_uniform_apply_pressure (uniformgrid_fluid.cu:239-260)
  void apply_pressure() {
    const R alpha = (R)0.5f * ph.rdx;
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++) {
          const size_t i = idx3(x, y, z);
          const size_t il = x > 0 ? i - 1 : i, ir = x < gx - 1 ? i + 1 : i;
          const size_t id = y > 0 ? i - gx : i, iu = y < gy - 1 ? i + gx : i;
          const size_t ib = z > 0 ? i - (size_t)gx * gy : i, iff = z < gz - 1 ? i + (size_t)gx * gy : i;
          const R pc = p[i];
          v[0][i] = v[0][i] - alpha * (w[ir] * (p[ir] - pc) + w[il] * (pc - p[il]));
          v[1][i] = v[1][i] - alpha * (w[iu] * (p[iu] - pc) + w[id] * (pc - p[id]));
          v[2][i] = v[2][i] - alpha * (w[iff] * (p[iff] - pc) + w[ib] * (pc - p[ib]));
        }
  }
  // With ref_compat the reference's 2 pairs at the coarsest level and 1 pair
  // on finer levels (fluid_simulation_uniform.cu:96-124); otherwise
  // jacobi_iters sweeps per level.
  int project() override {
    calc_divergence();
    for (int l = 1; l < levels; l++) restrict_level(l);
    const int top_pairs = P.ref_compat ? 2 : P.jacobi_iters / 2;
    const int pairs = P.ref_compat ? 1 : P.jacobi_iters / 2;
    for (int i = 0; i < top_pairs; i++) {
      jacobi(levels - 1, p, pt);
      jacobi(levels - 1, pt, p);
    }
    for (int l = levels - 2; l >= 0; l--) {
      prolongate(l);
      for (int i = 0; i < pairs; i++) {
        jacobi(l, p, pt);
        jacobi(l, pt, p);
      }
    }
    apply_pressure();
    return DCG_OK;
  }
  // projectLocal (fluid_simulation_uniform.cu:126-135): 5 pairs on level 0.
  int project_local() override {
    calc_divergence();
    const int pairs = P.ref_compat ? 5 : P.jacobi_iters / 2;
    for (int i = 0; i < pairs; i++) {
      jacobi(0, p, pt);
      jacobi(0, pt, p);
    }
    apply_pressure();
    return DCG_OK;
  }
  int add_noise(uint64_t seed, float amp) override {
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < gz; z++)
      for (int y = 0; y < gy; y++)
        for (int x = 0; x < gx; x++)
          for (int d = 0; d < 3; d++)
            v[d][idx3(x, y, z)] = v[d][idx3(x, y, z)] + (R)(amp * noise_unit(seed, x, y, z, 0, d));
    return DCG_OK;
  }
  std::vector<R> *field_ptr(int f) {
    switch (f) {
      case DCG_FIELD_DENSITY: return &q[0];
      case DCG_FIELD_VEL_X: return &v[0];
      case DCG_FIELD_VEL_Y: return &v[1];
      case DCG_FIELD_VEL_Z: return &v[2];
      case DCG_FIELD_FLUIDITY: return &w;
      case DCG_FIELD_PRESSURE: return &p;
      case DCG_FIELD_PRESSURE_TMP: return &pt;
      case DCG_FIELD_DIVERGENCE: return &dv;
      case DCG_FIELD_TEMPERATURE: return nq > 1 ? &q[1] : nullptr;
      case DCG_FIELD_VAPOR: return nq > 2 ? &q[2] : nullptr;
    }
    return nullptr;
  }
  // Uniform fields are exchanged at the finest level (first gx*gy*gz entries).
  int get_field(int f, double *dst) override {
    auto *fp = field_ptr(f);
    if (!fp) return fail(DCG_E_NOT_FOUND, "no such field");
    for (size_t i = 0; i < nc; i++) dst[i] = (double)(*fp)[i];
    return DCG_OK;
  }
  int set_field(int f, const double *src) override {
    auto *fp = field_ptr(f);
    if (!fp) return fail(DCG_E_NOT_FOUND, "no such field");
    for (size_t i = 0; i < nc; i++) (*fp)[i] = (R)src[i];
    return DCG_OK;
  }
  int get_dense(int f, double *dst) override { return get_field(f, dst); }
  // ---------------- renderer samplers (uniformgrid_rendering.cu:5-52) ----------------
  struct Sampler {
    const UG &u;
    void sample(V3<R> p, bool precise, March<R> &a) const {
      if (!precise) {
        a.ix = clampi((int)p.x, 0, u.gx - 1);
        a.iy = clampi((int)p.y, 0, u.gy - 1);
        a.iz = clampi((int)p.z, 0, u.gz - 1);
        const size_t c = u.idx3(a.ix, a.iy, a.iz);
        for (int k = 0; k < 8; k++) a.idx[k] = c;
        a.fx = a.fy = a.fz = 0;
        a.density = u.q[0][c];
        return;
      }
      const R x = p.x - (R)0.5f, y = p.y - (R)0.5f, z = p.z - (R)0.5f;
      const R xf = std::floor(x), yf = std::floor(y), zf = std::floor(z);
      a.ix = (int)xf; a.iy = (int)yf; a.iz = (int)zf;
      a.fx = x - xf; a.fy = y - yf; a.fz = z - zf;
      const int x0 = clampi(a.ix, 0, u.gx - 1), y0 = clampi(a.iy, 0, u.gy - 1), z0 = clampi(a.iz, 0, u.gz - 1);
      const size_t xs = a.ix < u.gx - 1 ? 1 : 0, ys = a.iy < u.gy - 1 ? (size_t)u.gx : 0,
                   zs = a.iz < u.gz - 1 ? (size_t)u.gx * u.gy : 0;
      a.idx[0] = u.idx3(x0, y0, z0);
      a.idx[1] = a.idx[0] + zs;
      a.idx[2] = a.idx[0] + ys;
      a.idx[3] = a.idx[1] + ys;
      a.idx[4] = a.idx[0] + xs;
      a.idx[5] = a.idx[4] + zs;
      a.idx[6] = a.idx[4] + ys;
      a.idx[7] = a.idx[6] + zs;
      a.density = interp(a, [&](size_t c) { return u.q[0][c]; });
    }
    R vel_len(const March<R> &a) const {
      const R vx = interp(a, [&](size_t c) { return u.v[0][c]; });
      const R vy = interp(a, [&](size_t c) { return u.v[1][c]; });
      const R vz = interp(a, [&](size_t c) { return u.v[2][c]; });
      return std::sqrt(vx * vx + vy * vy + vz * vz);
    }
    R fluid(const March<R> &a) const { return interp(a, [&](size_t c) { return u.w[c]; }); }
  };
  int render(const dcg_render_params &rp, double *out) const override {
    Sampler S{*this};
    Marcher<R, Sampler>{S, ph, rp}.image(out);
    return DCG_OK;
  }

  void info(dcg_info *i) const override {
    std::memset(i, 0, sizeof(*i));
    i->mode = DCG_MODE_UNIFORM;
    i->levels = levels;
    i->n_scalars = nq;
    i->num_cells = (int64_t)nc;
  }
  // k_uniform_debug_stats (uniformgrid_structure.cu:33-43): sum rho * w.
  int stats(dcg_stats *st) override {
    std::memset(st, 0, sizeof(*st));
    double mass = 0;
    for (size_t i = 0; i < nc; i++) mass += (double)q[0][i] * (double)w[i];
    st->leaf_cells[0] = (int64_t)nc;
    st->active_cells = (int64_t)nc;
    st->mass = mass;
    st->steps = steps;
    return DCG_OK;
  }
};

}  // namespace

struct dcgo_sim {
  std::unique_ptr<Base> impl;
  DC<float> *dcf = nullptr;
  DC<double> *dcd = nullptr;
  std::string err;
};

template <typename F> static int with_dc(dcgo_sim *s, F f) {
  if (!s) return DCG_E_INVALID;
  if (s->dcf) return f(*s->dcf);
  if (s->dcd) return f(*s->dcd);
  return DCG_E_INVALID;
}

extern "C" {

int dcgo_create(const dcg_params *params, int32_t mode, int32_t precision, dcgo_sim **out) {
  if (!params || !out) return DCG_E_INVALID;
  *out = nullptr;
  auto *s = new dcgo_sim();
  int rc;
  if (mode == DCG_MODE_ADAPTIVE) {
    if (precision == 0) {
      auto *d = new DC<float>();
      d->prec = 0;
      s->impl.reset(d);
      s->dcf = d;
      rc = d->create(*params);
    } else {
      auto *d = new DC<double>();
      d->prec = 1;
      s->impl.reset(d);
      s->dcd = d;
      rc = d->create(*params);
    }
  } else if (mode == DCG_MODE_UNIFORM) {
    if (precision == 0) {
      auto *u = new UG<float>();
      s->impl.reset(u);
      rc = u->create(*params);
    } else {
      auto *u = new UG<double>();
      s->impl.reset(u);
      rc = u->create(*params);
    }
  } else {
    delete s;
    return DCG_E_INVALID;
  }
  if (rc) {
    delete s;
    return rc;
  }
  *out = s;
  return DCG_OK;
}
int dcgo_destroy(dcgo_sim *s) {
  delete s;
  return DCG_OK;
}
int dcgo_reset(dcgo_sim *s) { return s ? s->impl->reset() : DCG_E_INVALID; }
int dcgo_step(dcgo_sim *s, int32_t n) { return s ? s->impl->step(n) : DCG_E_INVALID; }
int dcgo_advect_velocity(dcgo_sim *s) { return s ? s->impl->advect_velocity() : DCG_E_INVALID; }
int dcgo_adapt(dcgo_sim *s) { return s ? s->impl->adapt() : DCG_E_INVALID; }
int dcgo_project(dcgo_sim *s) { return s ? s->impl->project() : DCG_E_INVALID; }
int dcgo_project_local(dcgo_sim *s) { return s ? s->impl->project_local() : DCG_E_INVALID; }
int dcgo_advect_scalars(dcgo_sim *s) { return s ? s->impl->advect_scalars() : DCG_E_INVALID; }
int dcgo_add_velocity_noise(dcgo_sim *s, uint64_t seed, float amplitude) {
  return s ? s->impl->add_noise(seed, amplitude) : DCG_E_INVALID;
}
int dcgo_set_threads(int32_t n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
  return DCG_OK;
}
int dcgo_get_info(const dcgo_sim *s, dcg_info *info) {
  if (!s || !info) return DCG_E_INVALID;
  s->impl->info(info);
  return DCG_OK;
}
const char *dcgo_last_error_string(const dcgo_sim *s) { return s ? s->impl->err.c_str() : "null handle"; }
int dcgo_get_field(dcgo_sim *s, int32_t field, double *dst) {
  return s && dst ? s->impl->get_field(field, dst) : DCG_E_INVALID;
}
int dcgo_set_field(dcgo_sim *s, int32_t field, const double *src) {
  return s && src ? s->impl->set_field(field, src) : DCG_E_INVALID;
}
int dcgo_get_dense(dcgo_sim *s, int32_t field, double *dst) {
  return s && dst ? s->impl->get_dense(field, dst) : DCG_E_INVALID;
}
int dcgo_get_topology(dcgo_sim *s, int32_t *pos, uint32_t *parent, uint32_t *child,
                      uint8_t *flags, int64_t *load, int64_t *move_limit) {
  return with_dc(s, [&](auto &d) {
    for (int64_t b = 0; b < d.B; b++) {
      if (pos) {
        pos[4 * b] = d.bx[b]; pos[4 * b + 1] = d.by[b]; pos[4 * b + 2] = d.bz[b];
        pos[4 * b + 3] = d.lvl[b] == FREE ? -1 : (int32_t)d.lvl[b];
      }
      if (parent) parent[b] = d.parent[b] == NF ? 0xFFFFFFFFu : (uint32_t)d.parent[b];
      if (child)
        for (int c = 0; c < 8; c++)
          child[8 * b + c] = d.child[8 * b + c] == NF ? 0xFFFFFFFFu : (uint32_t)d.child[8 * b + c];
      if (flags) flags[b] = d.flags[b];
    }
    for (int l = 0; l < d.levels; l++) {
      if (load) load[l] = d.load[l];
      if (move_limit) move_limit[l] = d.moveLimit[l];
    }
    return DCG_OK;
  });
}
int dcgo_set_topology(dcgo_sim *s, const int32_t *pos, const uint32_t *parent,
                      const uint32_t *child, const int64_t *load, const int64_t *move_limit) {
  return with_dc(s, [&](auto &d) {
    for (int64_t b = 0; b < d.B; b++) {
      if (pos) {
        d.bx[b] = pos[4 * b]; d.by[b] = pos[4 * b + 1]; d.bz[b] = pos[4 * b + 2];
        d.lvl[b] = pos[4 * b + 3] < 0 ? FREE : (uint8_t)pos[4 * b + 3];
      }
      if (parent) d.parent[b] = parent[b] == 0xFFFFFFFFu ? NF : (int64_t)parent[b];
      if (child)
        for (int c = 0; c < 8; c++)
          d.child[8 * b + c] = child[8 * b + c] == 0xFFFFFFFFu ? NF : (int64_t)child[8 * b + c];
      d.flags[b] = 0;
    }
    for (int l = 0; l < d.levels; l++) {
      if (load) d.load[l] = load[l];
      if (move_limit) d.moveLimit[l] = move_limit[l];
    }
    d.rebuild_hash();
    d.rebuild_apron_fresh();
    return DCG_OK;
  });
}
int dcgo_set_apron(dcgo_sim *s, const int64_t *src) {
  return with_dc(s, [&](auto &d) {
    std::memcpy(d.apron.data(), src, d.apron.size() * sizeof(int64_t));
    return DCG_OK;
  });
}
int dcgo_get_apron(dcgo_sim *s, int64_t *dst) {
  return with_dc(s, [&](auto &d) {
    for (int64_t b = 0; b < d.B; b++)
      for (int a = 0; a < AV; a++)
        dst[(size_t)b * AV + a] = d.lvl[b] == FREE ? -1 : d.apron[(size_t)b * AV + a];
    return DCG_OK;
  });
}
int64_t dcgo_apron_mismatches(dcgo_sim *s) {
  int64_t n = -1;
  with_dc(s, [&](auto &d) {
    n = d.apron_mismatches();
    return DCG_OK;
  });
  return n;
}
int dcgo_get_last_adapt(dcgo_sim *s, int64_t *moves, int64_t *n_moves, int64_t *refines,
                        int64_t *n_refines) {
  return with_dc(s, [&](auto &d) {
    if (n_moves) *n_moves = (int64_t)d.lastMoves.size() / 2;
    if (n_refines) *n_refines = (int64_t)d.lastRefines.size() / 2;
    if (moves) std::copy(d.lastMoves.begin(), d.lastMoves.end(), moves);
    if (refines) std::copy(d.lastRefines.begin(), d.lastRefines.end(), refines);
    return DCG_OK;
  });
}
int dcgo_adapt_replay(dcgo_sim *s, const int64_t *moves, int64_t n_moves, const int64_t *refines,
                      int64_t n_refines) {
  return with_dc(s, [&](auto &d) { return d.replay(moves, n_moves, refines, n_refines); });
}
int dcgo_get_scores(dcgo_sim *s, float *subblock, float *block) {
  return with_dc(s, [&](auto &d) {
    d.calc_subblock_scores();
    d.accumulate_subblock_scores();
    if (subblock) std::copy(d.ss.begin(), d.ss.begin() + d.B * 8, subblock);
    if (block) std::copy(d.bs.begin(), d.bs.end(), block);
    return DCG_OK;
  });
}
int dcgo_set_emission(dcgo_sim *s, const double *src) {
  return s && src ? s->impl->set_emission(src) : DCG_E_INVALID;
}
int dcgo_set_heightmap(dcgo_sim *s, const float *heights, int32_t nx, int32_t nz) {
  return s ? s->impl->set_heightmap(heights, nx, nz) : DCG_E_INVALID;
}
int dcgo_get_stats(dcgo_sim *s, dcg_stats *st) { return s && st ? s->impl->stats(st) : DCG_E_INVALID; }
int dcgo_render(dcgo_sim *s, const dcg_render_params *rp, double *rgba) {
  if (!s || !rp || !rgba || rp->width <= 0 || rp->height <= 0 || rp->aa_samples < 1) return DCG_E_INVALID;
  return s->impl->render(*rp, rgba);
}
int dcgo_adjoint_step(dcgo_sim *s, const double *lam_in, double *lam_out, double *lam_em) {
  if (!lam_in || !lam_out) return DCG_E_INVALID;
  return with_dc(s, [&](auto &d) {
    d.adjoint_step(lam_in, lam_out, lam_em);
    return DCG_OK;
  });
}
int dcgo_adjoint_step_full(dcgo_sim *s, const double *lam_in, double *lam_out, double *lam_em, const int64_t *moves,
                           int64_t n_moves, const int64_t *refines, int64_t n_refines) {
  if (!s || !lam_in || !lam_out) return DCG_E_INVALID;
  return with_dc(s, [&](auto &d) { return d.adjoint_step_full(lam_in, lam_out, lam_em, moves, n_moves, refines, n_refines); });
}
int dcgo_adjoint_dense(dcgo_sim *s, const double *lam_dense, double *lam_cells) {
  if (!lam_dense || !lam_cells) return DCG_E_INVALID;
  return with_dc(s, [&](auto &d) {
    d.adjoint_dense(lam_dense, lam_cells);
    return DCG_OK;
  });
}
int dcgo_copy_state(dcgo_sim *dst, const dcgo_sim *src) {
  if (!dst || !src) return DCG_E_INVALID;
  if (dst->dcd && src->dcd) dst->dcd->copy_state_from(*src->dcd);
  else if (dst->dcf && src->dcf) dst->dcf->copy_state_from(*src->dcf);
  else return DCG_E_INVALID;
  return DCG_OK;
}

}  // extern "C"
