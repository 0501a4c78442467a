// dcg_dev.cuh — device-side data layout and helpers of the GB300 DCGrid step.
//
// Layout in HBM (one simulation):
//   block table (SoA over the block pool of max_blocks entries)
//     pos[b]      int4  {x, y, z, level}   level-local cell coords, level -1 = free
//     parent[b]   u32   8*parentBlock + subblock, or NONE
//     child[8b+s] u32   child block of subblock s, or NONE
//     nbr[27b+d]  u32   neighbour of direction d (26 used, d=13 is the block):
//                       (leveldiff << 28) | block, or OUT (outside the domain)
//     flags[b]    u8    1 = moved, 2 = refined by the current adaptation
//   fields: float planes of 64*max_blocks cells, cell c of block b at 64*b + c,
//   c = subblock(x,y,z bits) * 8 + cell(x,y,z bits) as in the reference
//   (src/dcgrid/dcgrid_utils.cuh:67-81).
// The 26-entry neighbour table replaces the reference's 216-entry apron index
// table (src/dcgrid/dcgrid.h:22): an apron cell is resolved from its
// direction's neighbour block; a coarser neighbour is sampled by injection,
// the coarse cell that contains the apron cell (dcgrid_structure.cu:85-91).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace dcg {

constexpr int BW = 4, BV = 64, AW = 6;
constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr uint32_t OUT = 0xFFFFFFFFu;
constexpr uint32_t NBR_MASK = 0x0FFFFFFFu;
constexpr int MAXL = 16;
constexpr uint8_t MOVED = 1, REFINED = 2;

// device counters (adaptation bookkeeping), indices into Dev::ctr
enum : int {
  C_MOVES = 0,        // moves recorded so far in this adaptation
  C_REFINES = 1,      // refinements recorded
  C_TOUCHED = 2,      // moved + new blocks
  C_MOVE_LIMIT = 3,   // scratch: limit l of the level being matched
  C_MATCHES = 4,      // scratch: first failing pair of the level being matched
  C_NCAND = 5,        // scratch: candidate count of a compaction
  C_SELECT = 6,       // scratch: 1 when a level's refinement candidates outnumber its limit
  C_MOVE_BEGIN = 16,  // [16 + L]: first move of level L
  C_MOVE_END = 32,    // [32 + L]
  C_REF_BEGIN = 48,   // [48 + L]: first refinement creating blocks of level L
  C_REF_END = 64,     // [64 + L]
  C_LOAD0 = 80,       // [80 + L]: load of level L before this adaptation's refinements
  C_COUNT = 128
};

struct Geom {
  int gx, gy, gz, levels, sparse, nq, ref_compat, mixed;
  int dpass, gpad;  // FP64 defect-correction passes of the pressure solve
  long long B;
  long long full[MAXL], budget[MAXL], off[MAXL];
  int rx[MAXL], ry[MAXL], rz[MAXL];
};

struct Phys {
  float dt, dx, rdx;
  int inlet;
  float v_emit, d_emit, emit_radius;
  int solids;
  float sphere_r;
  int criterion;
  float refine_threshold, vort_t, grad_t;
  float buoy_a, buoy_b, t_amb;
  int src;
  float src_c[3], src_r, src_val[3];
  int wind;
  float wind_v[3];
  float ter_amp, ter_base, ter_freq, ter_pers;
  int ter_oct;
  unsigned ter_seed;
  int em_n;
  float em_band;
  const float *em;  // em_n^3 emission field (device), or null
  float src_jit;    // source temperature jitter amplitude
  unsigned src_seed;
  const float *hm;  // hm_nx * hm_nz terrain heightmap (device, x fastest), or null
  int hm_nx, hm_nz;
  float hm_sx, hm_sz;  // texels per finest cell: hm_nx / gx, hm_nz / gz
};

struct Dev {
  Geom g;
  Phys ph;
  int4 *pos;
  uint32_t *parent, *child, *nbr;
  uint8_t *flags;
  long long *load, *move_limit;
  float *q[3], *tq[3], *v[3], *tv[3];
  uint16_t *qh[3], *tqh[3];  // scalar storage when g.mixed != 0 (1 = BF16, 2 = FP16)
  float *w, *p, *pt, *div;
  float *ss, *bs;          // subblock / block scores (8B+1, B)
  uint32_t *moves;         // (block, dest) pairs
  int4 *mold;              // position of each moved block before its move
  uint32_t *refines;       // (subblock, new block) pairs
  uint32_t *touched;       // moved + new blocks
  long long *ctr;          // C_COUNT counters
  uint32_t *err;           // device error word
  double *red;             // reductions (stats)
  uint32_t *bar;           // grid barrier {arrivals, generation}
  uint32_t *epoch;         // per block: sweeps completed in the running level solve
  uint32_t *binfo;         // level solve: block descriptions of the running level (BI_WORDS words per block)
  float *rr, *e, *et;      // defect correction: residual, correction and its ping-pong plane
  double *dnorm;           // defect correction: FP64 ||r||^2, ||div||^2 per pass
};

// Scoped atomics of the grid barriers (PTX memory model): arrivals are
// acquire-release read-modify-writes, the release of the waiting CTAs a
// release add on the generation word, the wait an acquire load of it. Before
// the arrival, __syncthreads orders the CTA's writes before thread 0's release;
// after the wait, __syncthreads orders thread 0's acquire before the CTA's
// reads; so every write before the barrier is visible to every read after it.
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void red_add_release(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(unsigned *p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Bounded wait for the generation word to leave g: after `limit` polls (2^22
// by default) the CTA records DCG_DEVERR_TIMEOUT (8) in the error word and
// gives up.
constexpr unsigned kPollLimit = 1u << 22;
__device__ __forceinline__ void barrier_wait(const unsigned *gen, unsigned g, uint32_t *errw,
                                             unsigned limit = kPollLimit) {
  volatile unsigned *err = errw;
  unsigned spins = 0;
  while (ld_acquire(gen) == g) {
    __nanosleep(32);
    if (++spins > limit || (*err & 8u)) {
      atomicOr(errw, 8u);
      break;
    }
  }
}

// Two-level grid barrier: CTAs arrive on one of 16 group counters (separate
// 128-byte lines); the last of each group arrives on the top counter, and the
// last there releases everyone through the generation word. Same bounded wait
// and timeout rule as grid_barrier. Layout (u32, from bar + 64): [0]
// generation, [32*(1+g)] group g counter, [32*17] top counter.
__device__ inline void grid_barrier_tree(uint32_t *bar, uint32_t *errw, unsigned nctas) {
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned *tb = bar + 64;
    volatile unsigned *err = errw;
    if ((*err & 8u) == 0) {
      const unsigned g = ld_acquire(tb);
      const unsigned grp = blockIdx.x & 15u;
      const unsigned members = (nctas >> 4) + ((grp < (nctas & 15u)) ? 1u : 0u);
      const unsigned groups = nctas < 16u ? nctas : 16u;
      bool release = false;
      if (atom_add_acq_rel(tb + 32 * (1 + grp), 1u) == members - 1) {
        st_relaxed(tb + 32 * (1 + grp), 0u);
        if (atom_add_acq_rel(tb + 32 * 17, 1u) == groups - 1) {
          st_relaxed(tb + 32 * 17, 0u);
          release = true;
        }
      }
      if (release)
        red_add_release(tb, 1u);
      else
        barrier_wait(tb, g, errw);
    }
  }
  __syncthreads();
}
__device__ inline void grid_barrier_tree(const Dev &D, unsigned nctas) { grid_barrier_tree(D.bar, D.err, nctas); }

// Grid-wide barrier for cooperative launches (all CTAs co-resident). The wait
// is bounded: after 2^22 polls the CTA records DCG_DEVERR_TIMEOUT (8) in the
// error word and continues; once that bit is set every later barrier returns
// at once, so a broken barrier costs one bounded wait and never hangs the GPU.
__device__ inline void grid_barrier(uint32_t *bar, uint32_t *errw, unsigned nctas, unsigned limit = kPollLimit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *err = errw;
    if ((*err & 8u) == 0) {
      const unsigned g = ld_acquire(bar + 1);
      if (atom_add_acq_rel(bar, 1u) == nctas - 1) {
        st_relaxed(bar, 0u);
        red_add_release(bar + 1, 1u);
      } else {
        barrier_wait(bar + 1, g, errw, limit);
      }
    }
  }
  __syncthreads();
}
__device__ inline void grid_barrier(const Dev &D, unsigned nctas) { grid_barrier(D.bar, D.err, nctas); }

// ---------------------------------------------------------------- index math
__host__ __device__ inline int spread2(int d, int off) { return ((d & 1) | ((d << 2) & 8)) << off; }
__host__ __device__ inline int local_of(int x, int y, int z) {
  return spread2(x, 2) + spread2(y, 1) + spread2(z, 0);
}
__host__ __device__ inline void local_xyz(int c, int &x, int &y, int &z) {
  const int sub = c >> 3;
  x = (((sub >> 2) & 1) << 1) | ((c >> 2) & 1);
  y = (((sub >> 1) & 1) << 1) | ((c >> 1) & 1);
  z = ((sub & 1) << 1) | (c & 1);
}
__host__ __device__ inline int clampi(int v, int a, int b) { return v < a ? a : (v > b ? b : v); }
__device__ inline float clampf_(float v, float a, float b) { return v < a ? a : (v > b ? b : v); }

__device__ inline uint32_t dense_index(const Geom &g, int x, int y, int z, int level) {
  return (uint32_t)(g.off[level] + ((long long)(x >> 2) * g.ry[level] + (y >> 2)) * g.rz[level] + (z >> 2));
}

// Finest allocated block at a level >= L that contains level-L cell q: the
// result of getBlockIndexDeep (dcgrid_utils.cuh:201-233), found here by
// descending the child pointers from the finest dense level.
__device__ inline uint32_t locate(const Dev &D, int qx, int qy, int qz, int L, int &lev) {
  const int S = D.g.sparse;
  if (L >= S) {
    lev = L;
    return dense_index(D.g, qx, qy, qz, L);
  }
  uint32_t b = dense_index(D.g, qx >> (S - L), qy >> (S - L), qz >> (S - L), S);
  int l = S;
  while (l > L) {
    const int4 bp = D.pos[b];
    const int sh = l - L;
    const int lx = (qx >> sh) - bp.x, ly = (qy >> sh) - bp.y, lz = (qz >> sh) - bp.z;
    const uint32_t ch = D.child[8u * b + ((((lx >> 1) & 1) << 2) | (((ly >> 1) & 1) << 1) | ((lz >> 1) & 1))];
    if (ch == NONE) break;
    b = ch;
    l--;
  }
  lev = l;
  return b;
}

// Descends from block b at level l to the finest block containing level-0 cell q.
__device__ inline uint32_t descend(const Dev &D, uint32_t b, int &l, int qx, int qy, int qz) {
  while (l > 0) {
    const int4 bp = D.pos[b];
    const int lx = (qx >> l) - bp.x, ly = (qy >> l) - bp.y, lz = (qz >> l) - bp.z;
    const uint32_t ch = D.child[8u * b + ((((lx >> 1) & 1) << 2) | (((ly >> 1) & 1) << 1) | ((lz >> 1) & 1))];
    if (ch == NONE) break;
    b = ch;
    l--;
  }
  return b;
}

// x / 6, correctly rounded, by the method for divisors known in advance of
// Brisebarre, Muller and Raina (IEEE Trans. Computers 53(8), 2004): q =
// RN(x z) with z = RN(1/6), the remainder x - 6q exactly by one FMA, then
// RN(q + r z). The method assumes no underflow: inputs below 2^-120 in
// magnitude (subnormal quotients, signed zeros) take the IEEE division.
// Infinite x gives a NaN remainder; q (= x / 6 for those) is returned then.
// The library's self-check (dcg_check_div6) compares the result with the
// IEEE division over every binary32 input.
__device__ __forceinline__ float div6(float x) {
  if (!(fabsf(x) >= 0x1p-120f) && x == x) return x / 6.f;
  const float z = 0x1.555556p-3f;
  const float q = __fmul_rn(x, z);
  const float r = fmaf(-q, 6.f, x);
  const float y = fmaf(r, z, q);
  return r == r ? y : q;
}

// div6 of both components with packed FP32x2 operations (each component the
// correctly rounded operation of div6's scalar form, so the results are div6's)
__device__ __forceinline__ float2 div6x2(float2 x) {
  const float2 z = make_float2(0x1.555556p-3f, 0x1.555556p-3f);
  const float2 q = __fmul2_rn(x, z);
  const float2 r = __ffma2_rn(q, make_float2(-6.f, -6.f), x);  // x - 6 q, exactly as fmaf(-q, 6, x)
  const float2 y = __ffma2_rn(r, z, q);
  float2 o;
  o.x = (!(fabsf(x.x) >= 0x1p-120f) && x.x == x.x) ? x.x / 6.f : (r.x == r.x ? y.x : q.x);
  o.y = (!(fabsf(x.y) >= 0x1p-120f) && x.y == x.y) ? x.y / 6.f : (r.y == r.y ? y.y : q.y);
  return o;
}

__device__ inline int dir_of(int a) { return a == 0 ? 0 : (a == AW - 1 ? 2 : 1); }

// Global cell index of apron cell (ax, ay, az) in [0,6)^3 of block b.
// Out-of-domain apron cells map to one of the block's own cells: the clamped
// cell, or - for blocks of hashed levels in compat mode - the cell the
// reference's refresh writes, SPREAD(clamp(a,1,4)) = clamp(a,1,4) mod 4
// (dcgrid_structure.cu:55-61).
__device__ inline unsigned long long apron_cell(const Dev &D, uint32_t b, int4 bp, int ax, int ay,
                                                int az) {
  const int d = dir_of(ax) * 9 + dir_of(ay) * 3 + dir_of(az);
  if (d == 13) return (unsigned long long)b * BV + local_of(ax - 1, ay - 1, az - 1);
  const uint32_t e = D.nbr[27u * b + d];
  if (e == OUT) {
    if (D.g.ref_compat && bp.w < D.g.sparse)
      return (unsigned long long)b * BV +
             local_of(clampi(ax, 1, BW) & 3, clampi(ay, 1, BW) & 3, clampi(az, 1, BW) & 3);
    return (unsigned long long)b * BV +
           local_of(clampi(ax, 1, BW) - 1, clampi(ay, 1, BW) - 1, clampi(az, 1, BW) - 1);
  }
  const uint32_t nb = e & NBR_MASK;
  const int k = (int)(e >> 28);
  const int cx = bp.x + ax - 1, cy = bp.y + ay - 1, cz = bp.z + az - 1;
  return (unsigned long long)nb * BV + local_of((cx >> k) & 3, (cy >> k) & 3, (cz >> k) & 3);
}

// The six Jacobi neighbours (L, R, D, U, B, F) of a cell, as global cell indices.
struct Nb6 {
  uint32_t i0, i1, i2, i3, i4, i5;
};
__device__ inline Nb6 jacobi_neighbours(const Dev &D, long long cell) {
  const uint32_t b = (uint32_t)(cell >> 6);
  const int4 bp = D.pos[b];
  int lx, ly, lz;
  local_xyz((int)(cell & 63), lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  Nb6 n;
  n.i0 = (uint32_t)apron_cell(D, b, bp, ax - 1, ay, az);
  n.i1 = (uint32_t)apron_cell(D, b, bp, ax + 1, ay, az);
  n.i2 = (uint32_t)apron_cell(D, b, bp, ax, ay - 1, az);
  n.i3 = (uint32_t)apron_cell(D, b, bp, ax, ay + 1, az);
  n.i4 = (uint32_t)apron_cell(D, b, bp, ax, ay, az - 1);
  n.i5 = (uint32_t)apron_cell(D, b, bp, ax, ay, az + 1);
  return n;
}
// ---------------------------------------------------------------- physics
// All float expressions below keep the operation order of the reference
// (src/utils/sim_utils.cu, src/sdf.cuh); the library is compiled with
// -fmad=false so no multiply-add is fused.
__device__ inline uint32_t hash32(uint32_t seed, int32_t i, int32_t k, int32_t o) {
  uint32_t h = seed ^ 0x9E3779B9u;
  h ^= (uint32_t)i * 0x85EBCA6Bu; h = (h ^ (h >> 15)) * 0x2C1B3C6Du;
  h ^= (uint32_t)k * 0xC2B2AE35u; h = (h ^ (h >> 13)) * 0x297A2D39u;
  h ^= (uint32_t)o * 0x27D4EB2Fu; h = (h ^ (h >> 16)) * 0x85EBCA77u;
  return h ^ (h >> 15);
}
__device__ inline unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ inline float noise_unit(unsigned long long seed, int x, int y, int z, int level, int comp) {
  unsigned long long h = mix64(seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(comp + 1));
  h = mix64(h ^ ((unsigned long long)(uint32_t)x * 0xD6E8FEB86659FD93ull));
  h = mix64(h ^ ((unsigned long long)(uint32_t)y * 0xA0761D6478BD642Full));
  h = mix64(h ^ ((unsigned long long)(uint32_t)z * 0xE7037ED1A0B428DBull));
  h = mix64(h ^ (unsigned long long)(uint32_t)level);
  const float u = (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
  return 2.0f * u - 1.0f;
}

// Bilinear sample of the heightmap at (x, z) in finest cells; texel centres
// at (i + 0.5) / hm_sx, edge texels extended. The coordinate is clamped to
// [-1, n] before the conversion to int, so far-away or NaN positions (render
// rays) index inside the map.
__device__ inline float heightmap_sample(const Phys &P, float x, float z) {
  const float u = fminf(fmaxf(x * P.hm_sx - 0.5f, -1.f), (float)P.hm_nx);
  const float v = fminf(fmaxf(z * P.hm_sz - 0.5f, -1.f), (float)P.hm_nz);
  const float iu = floorf(u), iv = floorf(v);
  const float fu = u - iu, fv = v - iv;
  const int i0 = min(max((int)iu, 0), P.hm_nx - 1), i1 = min(max((int)iu + 1, 0), P.hm_nx - 1);
  const int k0 = min(max((int)iv, 0), P.hm_nz - 1), k1 = min(max((int)iv + 1, 0), P.hm_nz - 1);
  const float h00 = P.hm[k0 * P.hm_nx + i0], h10 = P.hm[k0 * P.hm_nx + i1];
  const float h01 = P.hm[k1 * P.hm_nx + i0], h11 = P.hm[k1 * P.hm_nx + i1];
  const float a = h00 + (h10 - h00) * fu;
  const float b = h01 + (h11 - h01) * fu;
  return a + (b - a) * fv;
}

__device__ inline float terrain_height(const Phys &P, float x, float z) {
  if (P.hm) return P.ter_base + P.ter_amp * heightmap_sample(P, x, z);
  float sum = 0.f, amp = 1.f, norm = 0.f, f = P.ter_freq;
  for (int o = 0; o < P.ter_oct; o++) {
    const float u = x * f, v = z * f;
    const float iu = floorf(u), iv = floorf(v);
    const float fu = u - iu, fv = v - iv;
    const float su = fu * fu * (3.f - 2.f * fu);
    const float sv = fv * fv * (3.f - 2.f * fv);
    const int i0 = (int)iu, k0 = (int)iv;
    const float unit = 1.0f / 16777216.0f;
    const float a = (float)(hash32(P.ter_seed, i0, k0, o) >> 8) * unit;
    const float b = (float)(hash32(P.ter_seed, i0 + 1, k0, o) >> 8) * unit;
    const float c = (float)(hash32(P.ter_seed, i0, k0 + 1, o) >> 8) * unit;
    const float d = (float)(hash32(P.ter_seed, i0 + 1, k0 + 1, o) >> 8) * unit;
    const float ab = a + (b - a) * su;
    const float cd = c + (d - c) * su;
    sum = sum + amp * (ab + (cd - ab) * sv);
    norm = norm + amp;
    amp = amp * P.ter_pers;
    f = f * 2.f;
  }
  return P.ter_base + P.ter_amp * (sum / norm);
}

// sceneSDF (src/sdf.cuh:8-20) + terrain extension
__device__ inline float scene_sdf(const Geom &g, const Phys &P, float x, float y, float z) {
  float d = 3.402823466e+38f;
  if (P.solids & 1) {
    const float cx = (float)g.gx * 0.5f, cy = (float)g.gy * 0.45f, cz = (float)g.gz * 0.5f;
    const float r = P.sphere_r * P.rdx;
    const float ddx = x - cx, ddy = y - cy, ddz = z - cz;
    d = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz) - r;
  }
  if (P.solids & 2) {
    const float t = y - terrain_height(P, x, z);
    d = fminf(d, t);
  }
  return d;
}

// getCellFluidity (src/utils/sim_utils.cu:11-22)
__device__ inline float fluidity(const Geom &g, const Phys &P, int x, int y, int z, int scale) {
  if (P.solids == 0) return 1.f;
  const float s = (float)scale;
  const float d = scene_sdf(g, P, ((float)x + 0.5f) * s, ((float)y + 0.5f) * s, ((float)z + 0.5f) * s);
  const float overlap = clampf_(0.5f - d / (s * 1.73205f), 0.f, 1.f);
  return 1.f - overlap;
}

__device__ inline bool in_inlet(const Geom &g, const Phys &P, int x, int y, int z, int scale) {
  if (!P.inlet || y >= 0) return false;
  const float a = (float)(x * scale) - 0.5f * (float)g.gx;
  const float b = (float)(z * scale) - 0.5f * (float)g.gz;
  return sqrtf(a * a + b * b) < P.emit_radius * P.rdx;
}
__device__ inline bool outside(const Geom &g, int x, int y, int z, int scale) {
  return x < 0 || y < 0 || z < 0 || x * scale >= g.gx || y * scale >= g.gy || z * scale >= g.gz;
}
__device__ inline bool yz_inside(const Geom &g, int y, int z, int scale) {
  return y >= 0 && z >= 0 && y * scale < g.gy && z * scale < g.gz;
}
// velocityBndCond (sim_utils.cu:24-39) + wind extension
__device__ inline void vel_bc(const Geom &g, const Phys &P, float &vx, float &vy, float &vz, int x,
                              int y, int z, int scale) {
  if (in_inlet(g, P, x, y, z, scale)) {
    vx = 0.f; vy = P.v_emit; vz = 0.f;
    return;
  }
  if (P.wind && yz_inside(g, y, z, scale)) {
    if (x < 0) { vx = P.wind_v[0]; vy = P.wind_v[1]; vz = P.wind_v[2]; return; }
    if (x * scale >= g.gx) return;
  }
  if (outside(g, x, y, z, scale)) vx = vy = vz = 0.f;
}
// component `comp` of vel_bc alone (each output component of vel_bc depends
// only on its own input component)
__device__ inline float vel_bc1(const Geom &g, const Phys &P, float v, int comp, int x, int y, int z,
                                int scale) {
  if (in_inlet(g, P, x, y, z, scale)) return comp == 1 ? P.v_emit : 0.f;
  if (P.wind && yz_inside(g, y, z, scale)) {
    if (x < 0) return P.wind_v[comp];
    if (x * scale >= g.gx) return v;
  }
  if (outside(g, x, y, z, scale)) return 0.f;
  return v;
}
// densityBndCond (sim_utils.cu:41-55) + wind extension; scalar k
__device__ inline float q_bc(const Geom &g, const Phys &P, float q, int k, int x, int y, int z,
                             int scale) {
  if (in_inlet(g, P, x, y, z, scale)) return k == 0 ? P.d_emit : 0.f;
  if (P.wind && yz_inside(g, y, z, scale)) {
    if (x < 0) return 0.f;
    if (x * scale >= g.gx) return q;
  }
  if (outside(g, x, y, z, scale)) return 0.f;
  return q;
}
__device__ inline bool in_source(const Phys &P, int x, int y, int z, int scale) {
  if (!P.src) return false;
  const float s = (float)scale;
  const float cx = ((float)x + 0.5f) * s - P.src_c[0];
  const float cy = ((float)y + 0.5f) * s - P.src_c[1];
  const float cz = ((float)z + 0.5f) * s - P.src_c[2];
  return cx * cx + cy * cy + cz * cz < P.src_r * P.src_r;
}

// Value a source cell takes for scalar k: the temperature (k = 1) with the
// seeded per-cell jitter of the cell's level-local position.
__device__ inline float src_value_at(const Phys &P, int k, int x, int y, int z, int level) {
  if (k != 1 || P.src_jit == 0.f) return P.src_val[k];
  return P.src_val[1] + P.src_jit * noise_unit(P.src_seed, x, y, z, level, 7);
}

// Emission field (extension): trilinear sample of the em_n^3 field over
// x in [0,gx), y in [0,em_band), z in [0,gz) at the centre of cell (x,y,z) of
// a level with cell size `scale`; 0 outside the band.
__device__ inline float em_lerp(float a, float b, float t) { return a + (b - a) * t; }
__device__ inline float emission_at(const Geom &g, const Phys &P, int x, int y, int z, int scale) {
  if (P.em_n <= 0 || !P.em) return 0.f;
  const float s = (float)scale;
  const float yw = ((float)y + 0.5f) * s;
  if (!(yw < P.em_band)) return 0.f;
  const float xw = ((float)x + 0.5f) * s, zw = ((float)z + 0.5f) * s;
  const int n = P.em_n;
  const float top = (float)(n - 1);
  const float u = clampf_(xw * ((float)n / (float)g.gx) - 0.5f, 0.f, top);
  const float v = clampf_(yw * ((float)n / P.em_band) - 0.5f, 0.f, top);
  const float w = clampf_(zw * ((float)n / (float)g.gz) - 0.5f, 0.f, top);
  const int i0 = (int)floorf(u), j0 = (int)floorf(v), k0 = (int)floorf(w);
  const int i1 = i0 + 1 < n ? i0 + 1 : n - 1, j1 = j0 + 1 < n ? j0 + 1 : n - 1, k1 = k0 + 1 < n ? k0 + 1 : n - 1;
  const float fu = u - (float)i0, fv = v - (float)j0, fw = w - (float)k0;
  const float *E = P.em;
  auto at = [&](int i, int j, int k) { return E[((size_t)k * n + j) * n + i]; };
  const float e00 = em_lerp(at(i0, j0, k0), at(i1, j0, k0), fu);
  const float e10 = em_lerp(at(i0, j1, k0), at(i1, j1, k0), fu);
  const float e01 = em_lerp(at(i0, j0, k1), at(i1, j0, k1), fu);
  const float e11 = em_lerp(at(i0, j1, k1), at(i1, j1, k1), fu);
  return em_lerp(em_lerp(e00, e10, fv), em_lerp(e01, e11, fv), fw);
}

__device__ inline void set_err(const Dev &D, uint32_t bits) { atomicOr(D.err, bits); }

// ---------------------------------------------------------------- scalar storage
// Scalars are stored as FP32, BF16 (mode 1) or FP16 (mode 2); compute is FP32.
// Conversions to 16 bits round to nearest even.
__device__ inline float h16_to_f(uint16_t h, int mode) {
  return mode == 1 ? __bfloat162float(__ushort_as_bfloat16(h)) : __half2float(__ushort_as_half(h));
}
__device__ inline uint16_t f_to_h16(float v, int mode) {
  return mode == 1 ? __bfloat16_as_ushort(__float2bfloat16_rn(v)) : __half_as_ushort(__float2half_rn(v));
}
__device__ inline float q_ld(const Dev &D, int k, size_t i) {
  return D.g.mixed ? h16_to_f(D.qh[k][i], D.g.mixed) : D.q[k][i];
}
__device__ inline void q_st(const Dev &D, int k, size_t i, float v) {
  if (D.g.mixed) D.qh[k][i] = f_to_h16(v, D.g.mixed);
  else D.q[k][i] = v;
}
__device__ inline void tq_st(const Dev &D, int k, size_t i, float v) {
  if (D.g.mixed) D.tqh[k][i] = f_to_h16(v, D.g.mixed);
  else D.tq[k][i] = v;
}

// ---------------------------------------------------------------- staged block tiles
// block+halo tile strides: 52 (x) and 8 (y) put the 32 cells of either half
// of a block, and each of their six neighbour sets, in 32 distinct banks
#ifndef DCG_TILE_SX
#define DCG_TILE_SX 52
#endif
#ifndef DCG_TILE_SY
#define DCG_TILE_SY 8
#endif

// Lane layout of the staged block kernels (one warp per block of 64 cells):
// lane owns the z-adjacent cells c = 2*lane, 2*lane+1, the first at tile
// offset oA of a 6^3 tile with strides SX, SY, 1 (and +1 so that the pair is
// 8-byte aligned). Halo slot q = 0..2 of the lane is halo cell h = lane + 32q
// of the block's 96 face-halo cells, face f = h >> 4 (-x, +x, -y, +y, -z,
// +z, so slot q covers the two faces of axis q). hpk: tile position (9 bits)
// | cell in a same-level neighbour << 9 | clamped own cell << 15 | compat-
// quirk own cell << 21; hax: apron coordinates ax | ay << 4 | az << 8 | f << 12.
template <int SX, int SY>
__device__ __forceinline__ void halo_slots(int lane, int &oA, uint32_t hpk[3], uint32_t hax[3]) {
  {
    int x, y, z;
    local_xyz(2 * lane, x, y, z);
    oA = (x + 1) * SX + (y + 1) * SY + (z + 1) + 1;
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const int h = lane + 32 * q;
    const int f = h >> 4, i = 1 + ((h >> 2) & 3), j = 1 + (h & 3);
    const int side = (f & 1) ? AW - 1 : 0;
    const int ax = f < 2 ? side : i, ay = f < 2 ? i : (f < 4 ? side : j), az = f < 4 ? j : side;
    const int same = local_of((ax - 1) & 3, (ay - 1) & 3, (az - 1) & 3);
    const int self = local_of(clampi(ax, 1, BW) - 1, clampi(ay, 1, BW) - 1, clampi(az, 1, BW) - 1);
    const int quirk = local_of(clampi(ax, 1, BW) & 3, clampi(ay, 1, BW) & 3, clampi(az, 1, BW) & 3);
    hpk[q] = (uint32_t)(ax * SX + ay * SY + az + 1) | ((uint32_t)same << 9) | ((uint32_t)self << 15) |
             ((uint32_t)quirk << 21);
    hax[q] = (uint32_t)ax | ((uint32_t)ay << 4) | ((uint32_t)az << 8) | ((uint32_t)f << 12);
  }
}

// Cell index of halo slot (pk, ga) of block b from the neighbour-table entry e
// of the slot's face: apron_cell for a known face.
__device__ __forceinline__ size_t halo_cell(const Dev &D, uint32_t b, int4 bp, uint32_t e, uint32_t pk,
                                            uint32_t ga) {
  if (e == OUT) {
    const uint32_t li = (D.g.ref_compat && bp.w < D.g.sparse) ? (pk >> 21) & 63u : (pk >> 15) & 63u;
    return (size_t)b * BV + li;
  }
  const int k = (int)(e >> 28);
  uint32_t li = (pk >> 9) & 63u;
  if (k > 0) {
    const int cx = bp.x + (int)(ga & 15u) - 1, cy = bp.y + (int)((ga >> 4) & 15u) - 1,
              cz = bp.z + (int)((ga >> 8) & 15u) - 1;
    li = (uint32_t)local_of((cx >> k) & 3, (cy >> k) & 3, (cz >> k) & 3);
  }
  return (size_t)(e & NBR_MASK) * BV + li;
}

// ---------------------------------------------------------------- sampling
// Shared by the advection kernels and their adjoint, so both compute the same
// sample indices and weights.
struct Smp {
  unsigned long long idx[8];
  float wt[8];
  float wAcc;
  int x0, y0, z0, x1, y1, z1, scale;
};

// INIT_SAMPLE (src/dcgrid/dcgrid_fluid.cu:7-72): locate the finest block that
// holds the back-traced point, then trilinear weights x fluidity, renormalised.
// The block is found from the advected cell's own block through its neighbour
// table and child pointers (no hash probes); points more than one block away
// fall back to a descent from the finest dense level.
__device__ inline void sample_at(const Dev &D, uint32_t b0, int4 bp0, float pxw, float pyw, float pzw,
                                 Smp &s) {
  const int ix = clampi((int)floorf(pxw), 0, D.g.gx - 1);
  const int iy = clampi((int)floorf(pyw), 0, D.g.gy - 1);
  const int iz = clampi((int)floorf(pzw), 0, D.g.gz - 1);
  const int L0 = bp0.w;
  const int ddx = ((ix >> L0) >> 2) - (bp0.x >> 2);
  const int ddy = ((iy >> L0) >> 2) - (bp0.y >> 2);
  const int ddz = ((iz >> L0) >> 2) - (bp0.z >> 2);
  uint32_t b = NONE;
  int lev = L0;
  if (ddx >= -1 && ddx <= 1 && ddy >= -1 && ddy <= 1 && ddz >= -1 && ddz <= 1) {
    if ((ddx | ddy | ddz) == 0) {
      b = b0;
    } else {
      const uint32_t e = D.nbr[27u * b0 + (ddx + 1) * 9 + (ddy + 1) * 3 + (ddz + 1)];
      if (e != OUT) {
        b = e & NBR_MASK;
        lev = L0 + (int)(e >> 28);
      }
    }
    if (b != NONE && lev == L0) b = descend(D, b, lev, ix, iy, iz);
  }
  if (b == NONE) b = locate(D, ix, iy, iz, 0, lev);
  const int4 bp = (b == b0) ? bp0 : D.pos[b];
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
#pragma unroll
  for (int c = 0; c < 8; c++)
    s.idx[c] = apron_cell(D, b, bp, i + ((c >> 2) & 1), j + ((c >> 1) & 1), k + (c & 1));
  const float Dx = 1.f - dx, Dy = 1.f - dy, Dz = 1.f - dz;
  s.wt[0] = D.w[s.idx[0]] * Dx * Dy * Dz;
  s.wt[1] = D.w[s.idx[1]] * Dx * Dy * dz;
  s.wt[2] = D.w[s.idx[2]] * Dx * dy * Dz;
  s.wt[3] = D.w[s.idx[3]] * Dx * dy * dz;
  s.wt[4] = D.w[s.idx[4]] * dx * Dy * Dz;
  s.wt[5] = D.w[s.idx[5]] * dx * Dy * dz;
  s.wt[6] = D.w[s.idx[6]] * dx * dy * Dz;
  s.wt[7] = D.w[s.idx[7]] * dx * dy * dz;
  s.wAcc = s.wt[0] + s.wt[1] + s.wt[2] + s.wt[3] + s.wt[4] + s.wt[5] + s.wt[6] + s.wt[7];
  const float wInv = 1.f / s.wAcc;
#pragma unroll
  for (int c = 0; c < 8; c++) s.wt[c] = s.wt[c] * wInv;
}

__device__ inline void corner_of(const Smp &s, int c, int &x, int &y, int &z) {
  x = (c & 4) ? s.x1 : s.x0;
  y = (c & 2) ? s.y1 : s.y0;
  z = (c & 1) ? s.z1 : s.z0;
}

// The sample's 2x2x2 corner box lies inside the domain: then no corner is in
// the inlet (y < 0), left of a wind inflow (x < 0) or outside, and the
// boundary conditions of every corner return the sampled values unchanged.
__device__ __forceinline__ bool box_inside(const Geom &g, const Smp &s) {
  return s.x0 >= 0 && s.y0 >= 0 && s.z0 >= 0 && s.x1 * s.scale < g.gx && s.y1 * s.scale < g.gy &&
         s.z1 * s.scale < g.gz;
}

// Back-trace (dcgrid_fluid.cu:115-122): (pos + .5) * scale - v * dt * rdx.
__device__ inline void back_trace(const Dev &D, int4 bp, int c, size_t cell, float &px, float &py,
                                  float &pz) {
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const float scale = (float)(1 << bp.w);
  const float alpha = D.ph.dt * D.ph.rdx;
  px = ((float)(bp.x + lx) + 0.5f) * scale - D.v[0][cell] * alpha;
  py = ((float)(bp.y + ly) + 0.5f) * scale - D.v[1][cell] * alpha;
  pz = ((float)(bp.z + lz) + 0.5f) * scale - D.v[2][cell] * alpha;
}

// ---------------------------------------------------------------- statistics
// k_dcgrid_debug_stats (dcgrid_structure.cu:224-251) for one cell of block b,
// plus mass and leaf counts, reduced per warp into D.red (every lane of the
// warp calls this; a warp covers half of one block).
// Statistics of one cell: for a leaf cell, scale * |residual| with the FP32
// arithmetic of k_dcgrid_debug_stats (dcgrid_structure.cu:224-251), and its
// mass rho * w * scale^3 (extension); returns the cell's level, -1 when the
// cell is not a leaf (both values 0 then).
__device__ inline int stats_vals(const Dev &D, long long b, int c, float &res, float &mass) {
  res = mass = 0.f;
  if (b >= D.g.B) return -1;
  const int4 bp = D.pos[b];
  const size_t cell = (size_t)b * BV + c;
  if (bp.w < 0 || D.child[cell >> 3] != NONE) return -1;
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  const int scale = 1 << bp.w;
  const float alpha = D.ph.rdx * D.ph.rdx / (float)(scale * scale);
  const float *P = D.p;
  const float pc = P[cell];
  const float pl = P[apron_cell(D, (uint32_t)b, bp, ax - 1, ay, az)];
  const float pr = P[apron_cell(D, (uint32_t)b, bp, ax + 1, ay, az)];
  const float pd = P[apron_cell(D, (uint32_t)b, bp, ax, ay - 1, az)];
  const float pu = P[apron_cell(D, (uint32_t)b, bp, ax, ay + 1, az)];
  const float pb = P[apron_cell(D, (uint32_t)b, bp, ax, ay, az - 1)];
  const float pf = P[apron_cell(D, (uint32_t)b, bp, ax, ay, az + 1)];
  const float r = D.div[cell] - (pl + pr + pd + pu + pb + pf - 6.f * pc) * alpha;
  res = (float)scale * fabsf(r);
  mass = q_ld(D, 0, cell) * D.w[cell] * (float)(scale * scale * scale);
  return bp.w;
}
// Warp totals of stats_vals (FP64 sums); every lane receives them. A warp
// covers half of one block, so all its leaf cells share one level (lvl, cnt
// leaf cells).
struct WarpStats {
  double res, mass;
  int lvl, cnt;
};
__device__ inline WarpStats warp_sum_stats(double res, double mass, int lev) {
  for (int o = 16; o > 0; o >>= 1) {
    res += __shfl_xor_sync(0xffffffffu, res, o);
    mass += __shfl_xor_sync(0xffffffffu, mass, o);
  }
  const unsigned leafmask = __ballot_sync(0xffffffffu, lev >= 0);
  WarpStats w;
  w.res = res;
  w.mass = mass;
  w.cnt = __popc(leafmask);
  w.lvl = __shfl_sync(0xffffffffu, lev, leafmask ? __ffs(leafmask) - 1 : 0);
  return w;
}
__device__ inline WarpStats stats_warp(const Dev &D, long long b, int c) {
  float r, m;
  const int lev = stats_vals(D, b, c, r, m);
  return warp_sum_stats((double)r, (double)m, lev);
}
// adds warp totals into the member's reduction slots (lane 0). A non-finite
// total means a leaf cell's pressure, divergence, density or fluidity is NaN
// or infinite (a NaN anywhere in the velocity or the other scalars reaches
// these within one step); it sets DCG_DEVERR_NAN (4) in the error word.
__device__ inline void stats_flush(const Dev &D, double res, double mass, int lvl, double cnt) {
  if ((threadIdx.x & 31) == 0) {
    if (!isfinite(res) || !isfinite(mass)) atomicOr(D.err, 4u);
    if (res != 0.0) atomicAdd(&D.red[0], res);
    if (mass != 0.0) atomicAdd(&D.red[1], mass);
    if (cnt != 0.0) atomicAdd(&D.red[2 + lvl], cnt);
  }
}
// statistics of one cell, one double atomic per warp and quantity
__device__ inline void stats_cell(const Dev &D, long long b, int c) {
  const WarpStats w = stats_warp(D, b, c);
  stats_flush(D, w.res, w.mass, w.lvl, (double)w.cnt);
}

}  // namespace dcg
