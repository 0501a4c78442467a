// k_topology.cu — block table construction, neighbour tables and the
// GPU-resident adaptation (scores -> device-side ranking -> moves ->
// refinements -> neighbour rebuild -> value propagation), plus statistics.
//
// The reference runs adaptation through host round trips (scores copied to
// the host, std::nth_element/std::sort, indices copied back,
// fluid_simulation_dcgrid.cu:348-483). Here every decision is made on the
// device from counters in device memory, so a whole step has a fixed launch
// sequence and can be captured in a CUDA graph.
#include <algorithm>
#include <cfloat>
#include <vector>

#include "dcg_kernels.h"

namespace dcg {

// ------------------------------------------------------------------ init
__global__ void __launch_bounds__(256) k_init_blocks(Dev D) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= D.g.B) return;
  D.pos[b] = make_int4(0, 0, 0, -1);
  D.parent[b] = NONE;
  D.flags[b] = 0;
#pragma unroll
  for (int c = 0; c < 8; c++) D.child[8 * b + c] = NONE;
}

// k_dcgrid_activate_level (dcgrid_structure.cu:104-178): dense levels are laid
// out in (x, y, z) order, z fastest; one thread per cell.
__global__ void __launch_bounds__(256) k_activate_level(Dev D, int level) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nb = (long long)D.g.rx[level] * D.g.ry[level] * D.g.rz[level];
  const long long t = gid >> 6;
  if (t >= nb) return;
  const int c = (int)(gid & 63);
  const int tz = (int)(t % D.g.rz[level]);
  const int ty = (int)((t / D.g.rz[level]) % D.g.ry[level]);
  const int tx = (int)(t / ((long long)D.g.rz[level] * D.g.ry[level]));
  const int px = BW * tx, py = BW * ty, pz = BW * tz;
  const long long b = D.g.off[level] + t;
  const int scale = 1 << level;
  if (c == 0) {
    D.pos[b] = make_int4(px, py, pz, level);
    if (level < D.g.levels - 1)
      D.parent[b] = 8u * dense_index(D.g, px / 2, py / 2, pz / 2, level + 1) +
                    (uint32_t)((px % (2 * BW)) + (py % (2 * BW)) / 2 + (pz % (2 * BW)) / 4);
    if (level - 1 >= D.g.sparse)
      for (int k = 0; k < 8; k++)
        D.child[8 * b + k] = dense_index(D.g, 2 * px + BW * ((k >> 2) & 1), 2 * py + BW * ((k >> 1) & 1),
                                         2 * pz + BW * (k & 1), level - 1);
  }
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const size_t cell = (size_t)b * BV + c;
  D.w[cell] = fluidity(D.g, D.ph, px + lx, py + ly, pz + lz, scale);
}

// Neighbour table: for each allocated block and each of its 26 directions,
// the finest block at the same or a coarser level that contains the
// neighbouring block position, or OUT. This equals what the reference's
// apron refresh (dcgrid_structure.cu:30-92) and activation (:104-178) store
// for the border apron cells of that direction.
__device__ __forceinline__ void build_nbr_body(const Dev &D, int only_if_touched, unsigned bx, unsigned gx) {
  if (only_if_touched && D.ctr[C_TOUCHED] == 0) return;
  const long long gid = (long long)bx * blockDim.x + threadIdx.x;
  const long long b = gid / 27;
  if (b >= D.g.B) return;
  const int d = (int)(gid % 27);
  const int4 bp = D.pos[b];
  if (bp.w < 0) return;
  uint32_t e;
  if (d == 13) {
    e = (uint32_t)b;
  } else {
    const int L = bp.w, scale = 1 << L;
    const int qx = bp.x + BW * (d / 9 - 1), qy = bp.y + BW * ((d / 3) % 3 - 1), qz = bp.z + BW * (d % 3 - 1);
    if (qx < 0 || qy < 0 || qz < 0 || qx * scale >= D.g.gx || qy * scale >= D.g.gy || qz * scale >= D.g.gz) {
      e = OUT;
    } else {
      int lev;
      const uint32_t nb = locate(D, qx, qy, qz, L, lev);
      e = ((uint32_t)(lev - L) << 28) | nb;
    }
  }
  D.nbr[27 * b + d] = e;
}
__global__ void __launch_bounds__(256) k_build_nbr(Dev D, int only_if_touched) { build_nbr_body(D, only_if_touched, blockIdx.x, gridDim.x); }

// The neighbour table after an adaptation. With ref_compat, the rules of the
// reference's apron refresh (k_dcgrid_refresh_apron_indices,
// dcgrid_structure.cu:30-92) applied to each direction's entry: a moved or
// new block looks all its neighbours up afresh; another block looks a
// direction up afresh when its neighbour there moved, and when that
// neighbour is coarser and was refined it takes the refined subblock's child
// (one level deeper, as the reference does even where a finer block now
// lies). The cells of one direction's apron region lie in one subblock of a
// coarser neighbour (block positions are multiples of 4 cells), so the
// reference's per-cell update is the same for the whole direction. Without
// ref_compat every entry is looked up afresh.
__device__ __forceinline__ void refresh_nbr_body(const Dev &D, unsigned bx, unsigned gx) {
  if (!D.g.ref_compat) {
    build_nbr_body(D, 1, bx, gx);
    return;
  }
  if (D.ctr[C_TOUCHED] == 0) return;
  const long long gid = (long long)bx * blockDim.x + threadIdx.x;
  const long long b = gid / 27;
  if (b >= D.g.B) return;
  const int d = (int)(gid % 27);
  const int4 bp = D.pos[b];
  if (bp.w < 0 || d == 13) return;
  uint32_t e = D.nbr[27 * b + d];
  bool fresh = (D.flags[b] & MOVED) != 0;
  if (!fresh && e != OUT) {
    const uint32_t nb = e & NBR_MASK;
    const int k = (int)(e >> 28);
    const uint8_t fl = D.flags[nb];
    if (fl & MOVED) {
      fresh = true;
    } else if ((fl & REFINED) && k > 0) {
      // a cell of the direction's region, at the neighbour's level
      const int dx = d / 9 - 1, dy = (d / 3) % 3 - 1, dz = d % 3 - 1;
      const int x = dx < 0 ? bp.x - 1 : (dx > 0 ? bp.x + BW : bp.x);
      const int y = dy < 0 ? bp.y - 1 : (dy > 0 ? bp.y + BW : bp.y);
      const int z = dz < 0 ? bp.z - 1 : (dz > 0 ? bp.z + BW : bp.z);
      const int4 np = D.pos[nb];
      const int lx = (x >> k) - np.x, ly = (y >> k) - np.y, lz = (z >> k) - np.z;
      const uint32_t c = D.child[8u * nb + (uint32_t)((((lx >> 1) & 1) << 2) | (((ly >> 1) & 1) << 1) | ((lz >> 1) & 1))];
      if (c != NONE) e = ((uint32_t)(k - 1) << 28) | c;
    }
  }
  if (fresh) {
    const int L = bp.w, scale = 1 << L;
    const int qx = bp.x + BW * (d / 9 - 1), qy = bp.y + BW * ((d / 3) % 3 - 1), qz = bp.z + BW * (d % 3 - 1);
    if (qx < 0 || qy < 0 || qz < 0 || qx * scale >= D.g.gx || qy * scale >= D.g.gy || qz * scale >= D.g.gz) {
      e = OUT;
    } else {
      int lev;
      const uint32_t nb = locate(D, qx, qy, qz, L, lev);
      e = ((uint32_t)(lev - L) << 28) | nb;
    }
  }
  D.nbr[27 * b + d] = e;
}
__global__ void __launch_bounds__(256) k_refresh_nbr(Dev D) { refresh_nbr_body(D, blockIdx.x, gridDim.x); }

// ------------------------------------------------------------------ scores
__device__ inline bool level_blocked(const Dev &D, int level) {
  return (level == 0 && D.load[0] == D.g.full[0]) ||
         (level > 0 && D.load[level - 1] == D.g.full[level - 1]);
}

// k_dcgrid_calc_subblock_scores (dcgrid_adaptation.cu:10-40), geometric score.
__device__ __forceinline__ float geo_score(const Dev &D, long long sb) {
  const long long b = sb >> 3;
  const int4 bp = D.pos[b];
  if (D.child[sb] != NONE || bp.w < 0 || level_blocked(D, bp.w)) return -FLT_MAX;
  const float sc = (float)(1 << bp.w);
  const float px = sc * ((float)bp.x + 2.f * (float)((sb >> 2) & 1) + 1.f);
  const float py = sc * ((float)bp.y + 2.f * (float)((sb >> 1) & 1) + 1.f);
  const float pz = sc * ((float)bp.z + 2.f * (float)(sb & 1) + 1.f);
  const float ddx = px - .5f * (float)D.g.gx, ddy = py - .45f * (float)D.g.gy, ddz = pz - .5f * (float)D.g.gz;
  const float dd = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
  return dd < .2f * (float)D.g.gx ? 0.f : (float)D.g.gx / dd;
}
__device__ __forceinline__ void scores_geo_body(const Dev &D, unsigned bx, unsigned gx) {
  const long long sb = (long long)bx * blockDim.x + threadIdx.x;
  if (sb >= 8 * D.g.B) {
    if (sb == 8 * D.g.B) D.ss[sb] = 0.f;
    return;
  }
  D.ss[sb] = geo_score(D, sb);
}
__global__ void __launch_bounds__(256) k_scores_geo(Dev D) { scores_geo_body(D, blockIdx.x, gridDim.x); }

// Field criterion (extension): per cell max(|curl v|/vort_t, |grad rho|/grad_t)
// with the central differences of k_dcgrid_calc_vorticity
// (dcgrid_fluid.cu:146-172); subblock score = max over its 8 cells, reduced
// with warp shuffles (a subblock is 8 consecutive lanes).
__device__ __forceinline__ bool subblock_blocked(const Dev &D, long long sb, int4 bp) {
  return D.child[sb] != NONE || bp.w < 0 || (bp.w >= 0 && level_blocked(D, bp.w));
}
__device__ __forceinline__ float field_cell_score(const Dev &D, long long b, int4 bp, int c) {
  int lx, ly, lz;
  local_xyz(c, lx, ly, lz);
  const int ax = lx + 1, ay = ly + 1, az = lz + 1;
  const int scale = 1 << bp.w;
  const float alpha = 0.5f * D.ph.rdx / (float)scale;
  const unsigned long long L = apron_cell(D, (uint32_t)b, bp, ax - 1, ay, az);
  const unsigned long long R = apron_cell(D, (uint32_t)b, bp, ax + 1, ay, az);
  const unsigned long long Dn = apron_cell(D, (uint32_t)b, bp, ax, ay - 1, az);
  const unsigned long long U = apron_cell(D, (uint32_t)b, bp, ax, ay + 1, az);
  const unsigned long long Bk = apron_cell(D, (uint32_t)b, bp, ax, ay, az - 1);
  const unsigned long long F = apron_cell(D, (uint32_t)b, bp, ax, ay, az + 1);
  const float *W = D.w;
  const float wl = W[L], wr = W[R], wd = W[Dn], wu = W[U], wb = W[Bk], wf = W[F];
  const float *V0 = D.v[0], *V1 = D.v[1], *V2 = D.v[2];
  const float ox = alpha * ((wu * V2[U] - wd * V2[Dn]) - (wf * V1[F] - wb * V1[Bk]));
  const float oy = alpha * ((wf * V0[F] - wb * V0[Bk]) - (wr * V2[R] - wl * V2[L]));
  const float oz = alpha * ((wr * V1[R] - wl * V1[L]) - (wu * V0[U] - wd * V0[Dn]));
  const float gxr = alpha * (q_ld(D, 0, R) - q_ld(D, 0, L));
  const float gyr = alpha * (q_ld(D, 0, U) - q_ld(D, 0, Dn));
  const float gzr = alpha * (q_ld(D, 0, F) - q_ld(D, 0, Bk));
  const float om = sqrtf(ox * ox + oy * oy + oz * oz);
  const float gr = sqrtf(gxr * gxr + gyr * gyr + gzr * gzr);
  const float a = om / D.ph.vort_t, bb = gr / D.ph.grad_t;
  return fmaxf(0.f, a < bb ? bb : a);
}
// max over the 8 lanes of a subblock group (lanes 8k..8k+7 of a warp)
__device__ __forceinline__ float max8(float m) {
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  return m;
}
__device__ __forceinline__ void scores_fields_body(const Dev &D, unsigned bx, unsigned gx) {
  const long long gid = (long long)bx * blockDim.x + threadIdx.x;
  const long long b = gid >> 6;
  if (b >= D.g.B) {
    if (gid == 64 * D.g.B) D.ss[8 * D.g.B] = 0.f;
    return;
  }
  const int c = (int)(gid & 63);
  const int4 bp = D.pos[b];
  const long long sb = (long long)b * 8 + (c >> 3);
  const bool blocked = subblock_blocked(D, sb, bp);
  const float m = max8(blocked ? 0.f : field_cell_score(D, b, bp, c));
  if ((c & 7) == 0) D.ss[sb] = blocked ? -FLT_MAX : m;
}
__global__ void __launch_bounds__(256) k_scores_fields(Dev D) { scores_fields_body(D, blockIdx.x, gridDim.x); }

// k_dcgrid_accumulate_subblock_scores (dcgrid_adaptation.cu:42-63); with
// ref_compat the reference's ninth summand s[8] is included.
__device__ __forceinline__ void block_scores_body(const Dev &D, unsigned bx, unsigned gx) {
  const long long b = (long long)bx * blockDim.x + threadIdx.x;
  if (b >= D.g.B) return;
  D.bs[b] = -FLT_MAX;
  const int level = D.pos[b].w;
  if (level < 0 || level_blocked(D, level)) return;
  const float *s = D.ss + 8 * b;
  if (s[0] > 0.f && s[1] > 0.f && s[2] > 0.f && s[3] > 0.f && s[4] > 0.f && s[5] > 0.f && s[6] > 0.f &&
      s[7] > 0.f) {
    float sum = s[0] + s[1] + s[2] + s[3] + s[4] + s[5] + s[6] + s[7];
    if (D.g.ref_compat) sum = sum + s[8];
    D.bs[b] = .125f * sum;
  }
}
__global__ void __launch_bounds__(256) k_block_scores(Dev D) { block_scores_body(D, blockIdx.x, gridDim.x); }

// ------------------------------------------------------------------ moves
// Move limit of one level (fluid_simulation_dcgrid.cu:376-385).
__device__ __forceinline__ void move_setup_body(const Dev &D, int L, unsigned bx, unsigned gx) {
  const long long d0 = D.g.budget[L], d1 = 8 * D.g.budget[L + 1];
  long long l = d0 < d1 ? d0 : d1;
  l = l < D.load[L] ? l : D.load[L];
  const long long freeL = D.g.full[L] - D.load[L];
  l = l < freeL ? l : freeL;
  if (D.move_limit[L] > 0) l = l < D.move_limit[L] ? l : D.move_limit[L];
  D.ctr[C_MOVE_LIMIT] = l;
  D.ctr[C_MATCHES] = l;
  D.ctr[C_MOVE_BEGIN + L] = D.ctr[C_MOVES];
  D.ctr[C_MOVE_END + L] = D.ctr[C_MOVES];
}
__global__ void k_move_setup(Dev D, int L) { move_setup_body(D, L, blockIdx.x, gridDim.x); }

// Sort keys: blocks ascending by score, negative scores last; subblocks
// descending by score. The sort is stable over index-ordered input, so
// equal keys stay in index order. Only the allocated prefix of each range is
// sorted (load[L] blocks, 8 load[L+1] subblocks): unallocated blocks score
// -FLT_MAX, whose key is the largest one, so in the stable order they follow
// every allocated entry in index order, where they already are.
__device__ __forceinline__ void keys_blocks_body(const Dev &D, int L, uint32_t *keys, uint32_t *vals, unsigned bx, unsigned gx) {
  if (D.ctr[C_MOVE_LIMIT] == 0) return;
  const long long i = (long long)bx * blockDim.x + threadIdx.x;
  if (i >= D.g.budget[L]) return;
  const long long b = D.g.off[L] + i;
  const float s = D.bs[b];
  keys[i] = s < 0.f ? 0xFFFFFFFFu : (__float_as_uint(s) & 0x7FFFFFFFu);
  vals[i] = (uint32_t)b;
}
__global__ void __launch_bounds__(256) k_keys_blocks(Dev D, int L, uint32_t *keys, uint32_t *vals) { keys_blocks_body(D, L, keys, vals, blockIdx.x, gridDim.x); }
__device__ __forceinline__ void keys_dests_body(const Dev &D, int L, uint32_t *keys, uint32_t *vals, unsigned bx, unsigned gx) {
  if (D.ctr[C_MOVE_LIMIT] == 0) return;
  const long long i = (long long)bx * blockDim.x + threadIdx.x;
  if (i >= 8 * D.g.budget[L + 1]) return;
  const long long sb = 8 * D.g.off[L + 1] + i;
  const float s = D.ss[sb];
  uint32_t u = s == 0.f ? 0u : __float_as_uint(s);
  u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);  // order-preserving map
  keys[i] = ~u;                                      // descending
  vals[i] = (uint32_t)sb;
}
__global__ void __launch_bounds__(256) k_keys_dests(Dev D, int L, uint32_t *keys, uint32_t *vals) { keys_dests_body(D, L, keys, vals, blockIdx.x, gridDim.x); }
// First pair that fails the reference's match condition (cu:410-418).
__device__ __forceinline__ void match_body(const Dev &D, const uint32_t *blocks, const uint32_t *dests, unsigned bx, unsigned gx) {
  const long long l = D.ctr[C_MOVE_LIMIT];
  for (long long m = (long long)bx * blockDim.x + threadIdx.x; m < l; m += (long long)gx * blockDim.x) {
    const float sb = D.bs[blocks[m]], sd = D.ss[dests[m]];
    if (!(sb >= 0.f && sd >= 0.f && sb < sd)) atomicMin(&D.ctr[C_MATCHES], m);
  }
}
__global__ void __launch_bounds__(256) k_match(Dev D, const uint32_t *blocks, const uint32_t *dests) { match_body(D, blocks, dests, blockIdx.x, gridDim.x); }
// Records the matched pairs and protects blocks from moving at the next
// level: with ref_compat the block of the candidate *after* each match, as
// the reference's loop does (cu:415-417); otherwise the destination's block.
__device__ __forceinline__ void commit_moves_body(const Dev &D, int L, const uint32_t *blocks, const uint32_t *dests, unsigned bx, unsigned gx) {
  const long long l = D.ctr[C_MOVE_LIMIT];
  if (l == 0) return;
  const long long matches = D.ctr[C_MATCHES];
  const long long base = D.ctr[C_MOVE_BEGIN + L];
  const long long d1 = 8 * D.g.budget[L + 1];
  for (long long m = (long long)bx * blockDim.x + threadIdx.x; m <= matches;
       m += (long long)gx * blockDim.x) {
    if (m < matches) {
      D.moves[2 * (base + m)] = blocks[m];
      D.moves[2 * (base + m) + 1] = dests[m];
    }
    if (D.g.ref_compat) {
      if (m >= 1 && m < d1) D.bs[dests[m] >> 3] = -FLT_MAX;
    } else if (m < matches) {
      D.bs[dests[m] >> 3] = -FLT_MAX;
    }
  }
  if (bx == 0 && threadIdx.x == 0) {
    D.move_limit[L] = (long long)(unsigned long long)((float)matches * 1.2f);
    D.ctr[C_MOVES] = base + matches;
    D.ctr[C_MOVE_END + L] = base + matches;
  }
}
__global__ void __launch_bounds__(256) k_commit_moves(Dev D, int L, const uint32_t *blocks, const uint32_t *dests) { commit_moves_body(D, L, blocks, dests, blockIdx.x, gridDim.x); }
// k_dcgrid_move_blocks (dcgrid_adaptation.cu:65-90), one level at a time from
// coarse to fine so a block moved into a block that itself moved takes its
// parent's new position.
__device__ __forceinline__ void apply_moves_body(const Dev &D, int L, uint32_t *prevs, unsigned bx, unsigned gx) {
  const long long beg = D.ctr[C_MOVE_BEGIN + L], end = D.ctr[C_MOVE_END + L];
  for (long long m = beg + (long long)bx * blockDim.x + threadIdx.x; m < end;
       m += (long long)gx * blockDim.x) {
    const uint32_t b = D.moves[2 * m], dest = D.moves[2 * m + 1];
    const uint32_t prev = D.parent[b];
    prevs[m] = prev;
    if (prev != NONE) D.child[prev] = NONE;
    D.child[dest] = b;
    D.parent[b] = dest;
    const uint32_t pb = dest >> 3;
    const int4 pp = D.pos[pb];
    const int4 old = D.pos[b];
    D.mold[m] = old;
    D.pos[b] = make_int4(2 * pp.x + BW * ((dest >> 2) & 1), 2 * pp.y + BW * ((dest >> 1) & 1),
                         2 * pp.z + BW * (dest & 1), old.w);
    D.flags[b] |= MOVED;
    D.flags[pb] |= REFINED;
    D.touched[m] = b;
  }
}
__global__ void __launch_bounds__(256) k_apply_moves(Dev D, int L, uint32_t *prevs) { apply_moves_body(D, L, prevs, blockIdx.x, gridDim.x); }

// Subblock scores after the moves (the reference recomputes every score,
// fluid_simulation_dcgrid.cu:436). A score depends on its block's position,
// its own child pointer, the level loads, the neighbour table and the field
// values; moves change only the positions of moved blocks and the child
// pointers of their previous and new parent subblocks. Recomputing those
// subblocks (10 per move: the moved block's 8, the old and the new parent
// subblock) gives exactly the scores of a full pass. The neighbour table is
// rebuilt only after the refinements, as the reference's apron indices are
// refreshed only then (dcgrid_structure.cu:30-92): until then a moved block
// reads the neighbours of its old place, so its cells in a coarser neighbour
// come from its position before the move (mold), as the stored apron
// indices give them.
__device__ __forceinline__ uint32_t rescore_target(const Dev &D, const uint32_t *prevs, long long t) {
  const long long m = t / 10;
  const int k = (int)(t - 10 * m);
  if (k < 8) return 8u * D.moves[2 * m] + (uint32_t)k;
  return k == 8 ? prevs[m] : D.moves[2 * m + 1];
}
__device__ __forceinline__ void rescore_body(const Dev &D, const uint32_t *prevs, unsigned bx, unsigned gx) {
  const long long ntask = 10 * D.ctr[C_MOVES];
  if (ntask == 0) return;
  if (D.ph.criterion == 0) {
    for (long long t = (long long)bx * blockDim.x + threadIdx.x; t < ntask; t += (long long)gx * blockDim.x) {
      const uint32_t sb = rescore_target(D, prevs, t);
      if (sb != NONE) D.ss[sb] = geo_score(D, sb);
    }
    return;
  }
  // field criterion: 8 lanes per subblock, 4 subblocks per warp pass
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)bx * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gx * blockDim.x) >> 5;
  for (long long tw = 4 * w0; tw < ntask; tw += 4 * nw) {
    const long long t = tw + (lane >> 3);
    const uint32_t sb = t < ntask ? rescore_target(D, prevs, t) : NONE;
    const long long b = sb == NONE ? 0 : (long long)(sb >> 3);
    // a moved block's own subblocks (targets 0-7 of its move): its old position
    const bool own = t < ntask && t - 10 * (t / 10) < 8;
    const int4 bp = sb == NONE ? make_int4(0, 0, 0, -1) : (own ? D.mold[t / 10] : D.pos[b]);
    const bool blocked = sb == NONE || subblock_blocked(D, sb, bp);
    const float m = max8(blocked ? 0.f : field_cell_score(D, b, bp, (int)(8 * (sb & 7) + (lane & 7))));
    if ((lane & 7) == 0 && sb != NONE) D.ss[sb] = blocked ? -FLT_MAX : m;
  }
}
__global__ void __launch_bounds__(256) k_rescore(Dev D, const uint32_t *prevs) { rescore_body(D, prevs, blockIdx.x, gridDim.x); }

// ------------------------------------------------------------ refinements
// Refinement limit of one parent level (fluid_simulation_dcgrid.cu:449-453).
__device__ __forceinline__ void refine_setup_body(const Dev &D, int L, unsigned bx, unsigned gx) {
  const unsigned long long a = (unsigned long long)(D.g.budget[L - 1] - D.load[L - 1]);
  const unsigned long long bb = (unsigned long long)(8 * D.load[L]) - (unsigned long long)D.load[L - 1];
  const long long limit = (long long)(a < bb ? a : bb);
  D.ctr[C_MOVE_LIMIT] = limit;
  D.ctr[C_REF_BEGIN + L - 1] = D.ctr[C_REFINES];
  D.ctr[C_REF_END + L - 1] = D.ctr[C_REFINES];
  D.ctr[C_LOAD0 + L - 1] = D.load[L - 1];
  D.ctr[C_NCAND] = 0;
  D.ctr[C_SELECT] = 0;
}
__global__ void k_refine_setup(Dev D, int L) { refine_setup_body(D, L, blockIdx.x, gridDim.x); }

constexpr int CMP_TILE = 2048;

// Compaction of flagged subblocks (stable, ascending index): tile counts,
// a single-CTA scan over tiles, then per-tile ranks.
__device__ inline bool cand_flag(const Dev &D, int L, long long i, const uint8_t *sel) {
  if (sel) return sel[8 * D.g.off[L] + i] != 0;
  return D.ss[8 * D.g.off[L] + i] > D.ph.refine_threshold;
}
__device__ __forceinline__ void cmp_count_body(const Dev &D, int L, const uint8_t *sel, uint32_t *tile_sums, unsigned bx, unsigned gx) {
  if (D.ctr[C_MOVE_LIMIT] == 0 || (sel && D.ctr[C_SELECT] == 0)) return;
  const long long n = 8 * D.g.budget[L];
  const long long base = (long long)bx * CMP_TILE;
  int cnt = 0;
  for (int r = 0; r < CMP_TILE / 256; r++) {
    const long long i = base + r * 256 + threadIdx.x;
    if (i < n && cand_flag(D, L, i, sel)) cnt++;
  }
  cnt = __reduce_add_sync(0xffffffffu, (unsigned)cnt);
  __shared__ int ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < 8; w++) t += ws[w];
    tile_sums[bx] = (uint32_t)t;
  }
}
__global__ void __launch_bounds__(256) k_cmp_count(Dev D, int L, const uint8_t *sel, uint32_t *tile_sums) { cmp_count_body(D, L, sel, tile_sums, blockIdx.x, gridDim.x); }
// first: the threshold compaction, which also decides whether the
// score-ordered selection is needed (C_SELECT); else the selection's
// compaction, which runs only then
__device__ __forceinline__ void cmp_scan_body(const Dev &D, uint32_t *tile_sums, long long ntiles, int first, unsigned bx, unsigned gx) {
  if (D.ctr[C_MOVE_LIMIT] == 0 || (!first && D.ctr[C_SELECT] == 0)) return;
  __shared__ uint32_t ws[32];
  __shared__ uint32_t carry_s;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long t0 = 0; t0 < ntiles; t0 += 1024) {
    const long long t = t0 + threadIdx.x;
    const uint32_t v = t < ntiles ? tile_sums[t] : 0;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t s = ws[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      ws[lane] = s;
    }
    __syncthreads();
    const uint32_t carry = carry_s;
    const uint32_t ex = carry + (warp ? ws[warp - 1] : 0) + x - v;
    if (t < ntiles) tile_sums[t] = ex;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = carry + ws[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    D.ctr[C_NCAND] = carry_s;
    // more candidates than the limit: only then does their score order matter
    if (first) D.ctr[C_SELECT] = (long long)carry_s > D.ctr[C_MOVE_LIMIT] ? 1 : 0;
  }
}
__global__ void __launch_bounds__(1024) k_cmp_scan(Dev D, uint32_t *tile_sums, long long ntiles, int first) { cmp_scan_body(D, tile_sums, ntiles, first, blockIdx.x, gridDim.x); }
__device__ __forceinline__ void cmp_scatter_body(const Dev &D, int L, const uint8_t *sel, const uint32_t *tile_sums, uint32_t *out, unsigned bx, unsigned gx) {
  if (D.ctr[C_MOVE_LIMIT] == 0 || (sel && D.ctr[C_SELECT] == 0)) return;
  __shared__ uint32_t ws[8];
  __shared__ uint32_t run_s;
  const long long n = 8 * D.g.budget[L];
  const long long base = (long long)bx * CMP_TILE;
  if (threadIdx.x == 0) run_s = tile_sums[bx];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int r = 0; r < CMP_TILE / 256; r++) {
    const long long i = base + r * 256 + threadIdx.x;
    const bool f = i < n && cand_flag(D, L, i, sel);
    const uint32_t bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) ws[warp] = __popc(bal);
    __syncthreads();
    uint32_t before = run_s;
    for (int w = 0; w < warp; w++) before += ws[w];
    if (f) out[before + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)(8 * D.g.off[L] + i);
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int w = 0; w < 8; w++) t += ws[w];
      run_s += t;
    }
    __syncthreads();
  }
}
__global__ void __launch_bounds__(256) k_cmp_scatter(Dev D, int L, const uint8_t *sel, const uint32_t *tile_sums, uint32_t *out) { cmp_scatter_body(D, L, sel, tile_sums, out, blockIdx.x, gridDim.x); }
// Score-ordered selection (ref_compat off): keys of the compacted candidates.
__device__ __forceinline__ void keys_cands_body(const Dev &D, const uint32_t *cand, uint32_t *keys, uint32_t *vals, long long nmax, unsigned bx, unsigned gx) {
  if (D.ctr[C_SELECT] == 0) return;  // every candidate is kept: no selection
  const long long n = D.ctr[C_NCAND];
  for (long long i = (long long)bx * blockDim.x + threadIdx.x; i < nmax; i += (long long)gx * blockDim.x) {
    if (i < n) {
      const float s = D.ss[cand[i]];
      uint32_t u = s == 0.f ? 0u : __float_as_uint(s);
      u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
      keys[i] = ~u;
      vals[i] = cand[i];
    } else {
      keys[i] = 0xFFFFFFFFu;  // pads sort after every candidate
      vals[i] = 0xFFFFFFFFu;
    }
  }
}
__global__ void __launch_bounds__(256) k_keys_cands(Dev D, const uint32_t *cand, uint32_t *keys, uint32_t *vals, long long nmax) { keys_cands_body(D, cand, keys, vals, nmax, blockIdx.x, gridDim.x); }
__device__ __forceinline__ void mark_selected_body(const Dev &D, const uint32_t *sorted, uint8_t *sel, unsigned bx, unsigned gx) {
  if (D.ctr[C_MOVE_LIMIT] == 0 || D.ctr[C_SELECT] == 0) return;
  const long long n = D.ctr[C_NCAND], limit = D.ctr[C_MOVE_LIMIT];
  const long long keep = n < limit ? n : limit;
  for (long long i = (long long)bx * blockDim.x + threadIdx.x; i < keep; i += (long long)gx * blockDim.x)
    sel[sorted[i]] = 1;
}
__global__ void __launch_bounds__(256) k_mark_selected(Dev D, const uint32_t *sorted, uint8_t *sel) { mark_selected_body(D, sorted, sel, blockIdx.x, gridDim.x); }
// Records the kept candidates of one level and assigns new block indices in
// ascending subblock order. ref_compat keeps the `limit` largest subblock
// indices (the reference's nth_element over indices, cu:464-466).
__device__ __forceinline__ void record_refines_body(const Dev &D, int L, const uint32_t *cand, int compat_tail, unsigned bx, unsigned gx) {
  const long long limit = D.ctr[C_MOVE_LIMIT];
  if (limit == 0) return;
  const long long n = D.ctr[C_NCAND];
  const long long keep = n < limit ? n : limit;
  const long long first = compat_tail ? n - keep : 0;
  const long long base = D.ctr[C_REF_BEGIN + L - 1];
  const long long load0 = D.ctr[C_LOAD0 + L - 1];
  for (long long r = (long long)bx * blockDim.x + threadIdx.x; r < keep; r += (long long)gx * blockDim.x) {
    D.refines[2 * (base + r)] = cand[first + r];
    D.refines[2 * (base + r) + 1] = (uint32_t)(D.g.off[L - 1] + load0 + r);
  }
  if (bx == 0 && threadIdx.x == 0) {
    D.ctr[C_REFINES] = base + keep;
    D.ctr[C_REF_END + L - 1] = base + keep;
  }
}
__global__ void __launch_bounds__(256) k_record_refines(Dev D, int L, const uint32_t *cand, int compat_tail) { record_refines_body(D, L, cand, compat_tail, blockIdx.x, gridDim.x); }
// k_dcgrid_refine_subblocks + insertBlock (dcgrid_adaptation.cu:145-178,
// dcgrid_utils.cuh:99-140) for every recorded refinement.
__device__ __forceinline__ void apply_refines_body(const Dev &D, unsigned bx, unsigned gx) {
  const long long nr = D.ctr[C_REFINES], nm = D.ctr[C_MOVES];
  for (long long m = (long long)bx * blockDim.x + threadIdx.x; m < nr; m += (long long)gx * blockDim.x) {
    const uint32_t sb = D.refines[2 * m], cb = D.refines[2 * m + 1];
    const uint32_t pb = sb >> 3;
    const int4 pp = D.pos[pb];
    const int cl = pp.w - 1;
    if (cl < 0 || (long long)cb >= D.g.off[cl] + D.g.budget[cl]) {
      set_err(D, 1u);
      D.touched[nm + m] = NONE;
      continue;
    }
    D.pos[cb] = make_int4(2 * pp.x + BW * ((sb >> 2) & 1), 2 * pp.y + BW * ((sb >> 1) & 1),
                          2 * pp.z + BW * (sb & 1), cl);
    D.parent[cb] = sb;
    D.child[sb] = cb;
    D.flags[pb] |= REFINED;
    D.flags[cb] |= MOVED;
    D.touched[nm + m] = cb;
  }
}
__global__ void __launch_bounds__(256) k_apply_refines(Dev D) { apply_refines_body(D, blockIdx.x, gridDim.x); }
__device__ __forceinline__ void finish_refines_body(const Dev &D, unsigned bx, unsigned gx) {
  for (int L = 1; L < D.g.levels; L++) {
    const long long n = D.ctr[C_REF_END + L - 1] - D.ctr[C_REF_BEGIN + L - 1];
    D.load[L - 1] += n;
  }
  D.ctr[C_TOUCHED] = D.ctr[C_MOVES] + D.ctr[C_REFINES];
}
__global__ void k_finish_refines(Dev D) { finish_refines_body(D, blockIdx.x, gridDim.x); }

// k_dcgrid_propagate_values (dcgrid_adaptation.cu:92-143): new or moved blocks
// of one level take 27/9/3/1 interpolations of their parent's apron.
__device__ __forceinline__ void propagate_body(const Dev &D, int level, unsigned bx, unsigned gx) {
  const long long nt = D.ctr[C_TOUCHED];
  const int c = threadIdx.x & 63;
  for (long long t = (long long)bx * 4 + (threadIdx.x >> 6); t < nt; t += (long long)gx * 4) {
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
    const unsigned long long i000 = apron_cell(D, pb, pbp, ax, ay, az);
    const unsigned long long i001 = apron_cell(D, pb, pbp, ax, ay, az + k);
    const unsigned long long i010 = apron_cell(D, pb, pbp, ax, ay + j, az);
    const unsigned long long i100 = apron_cell(D, pb, pbp, ax + i, ay, az);
    const unsigned long long i011 = apron_cell(D, pb, pbp, ax, ay + j, az + k);
    const unsigned long long i101 = apron_cell(D, pb, pbp, ax + i, ay, az + k);
    const unsigned long long i110 = apron_cell(D, pb, pbp, ax + i, ay + j, az);
    const unsigned long long i111 = apron_cell(D, pb, pbp, ax + i, ay + j, az + k);
    const size_t cell = (size_t)b * BV + c;
    auto tri = [&](const float *f) {
      return (27.f / 64.f) * f[i000] + (9.f / 64.f) * (f[i001] + f[i010] + f[i100]) +
             (3.f / 64.f) * (f[i011] + f[i101] + f[i110]) + (1.f / 64.f) * f[i111];
    };
    auto triq = [&](int k) {
      return (27.f / 64.f) * q_ld(D, k, i000) +
             (9.f / 64.f) * (q_ld(D, k, i001) + q_ld(D, k, i010) + q_ld(D, k, i100)) +
             (3.f / 64.f) * (q_ld(D, k, i011) + q_ld(D, k, i101) + q_ld(D, k, i110)) +
             (1.f / 64.f) * q_ld(D, k, i111);
    };
    float qv[3], vv[3];
    for (int kq = 0; kq < D.g.nq; kq++) qv[kq] = triq(kq);
    for (int d = 0; d < 3; d++) vv[d] = tri(D.v[d]);
    for (int kq = 0; kq < D.g.nq; kq++) q_st(D, kq, cell, qv[kq]);
    for (int d = 0; d < 3; d++) D.v[d][cell] = vv[d];
    D.w[cell] = fluidity(D.g, D.ph, x, y, z, 1 << level);
  }
}
__global__ void __launch_bounds__(256) k_propagate(Dev D, int level) { propagate_body(D, level, blockIdx.x, gridDim.x); }

static unsigned grid_for(long long n, int threads = 256) {
  return (unsigned)((n + threads - 1) / threads);
}

void launch_init_blocks(const Dev &D, cudaStream_t st) {
  k_init_blocks<<<grid_for(D.g.B), 256, 0, st>>>(D);
}
void launch_activate_level(const Dev &D, int level, cudaStream_t st) {
  const long long nb = (long long)D.g.rx[level] * D.g.ry[level] * D.g.rz[level];
  k_activate_level<<<grid_for(nb * 64), 256, 0, st>>>(D, level);
}
void launch_build_nbr(const Dev &D, bool only_if_touched, cudaStream_t st) {
  k_build_nbr<<<grid_for(D.g.B * 27), 256, 0, st>>>(D, only_if_touched ? 1 : 0);
}

static void launch_scores_staged(const Dev *d, int n, cudaStream_t st);
static void launch_scores(const Dev &D, cudaStream_t st) {
  if (D.ph.criterion == 0)
    k_scores_geo<<<grid_for(8 * D.g.B + 1), 256, 0, st>>>(D);
  else
    launch_scores_staged(&D, 1, st);
}

// A level whose budget covers its whole block grid is allocated in full when
// the simulation is created and keeps every block (blocks are never freed),
// so its move limit (free places at the level) and the refinement limit of
// the level above it (free blocks at the level) are 0: those passes change
// nothing and are not launched. (Their only writes are the pass's own
// scratch counters.)
static bool level_full(const Geom &g, int L) { return g.budget[L] == g.full[L]; }

// FluidSimulationDCGrid::adaptTopology (fluid_simulation_dcgrid.cu:320-346)
// as a fixed sequence of launches.
void launch_adapt(const Dev &D, const SortScratch &s, uint32_t *keys, uint32_t *vals, uint32_t *keys2,
                  uint32_t *vals2, int sms, cudaStream_t st) {
  const unsigned gs = (unsigned)(sms > 0 ? sms * 4 : 512);
  cudaMemsetAsync(D.ctr, 0, sizeof(long long) * C_COUNT, st);
  cudaMemsetAsync(D.flags, 0, (size_t)D.g.B, st);
  // moveBlocks
  launch_scores(D, st);
  k_block_scores<<<grid_for(D.g.B), 256, 0, st>>>(D);
  for (int L = 0; L < D.g.levels - 1; L++) {
    if (level_full(D.g, L)) continue;  // no free place at level L: no move (limit 0)
    const long long d0 = D.g.budget[L], d1 = 8 * D.g.budget[L + 1];
    k_move_setup<<<1, 1, 0, st>>>(D, L);
    k_keys_blocks<<<grid_for(d0), 256, 0, st>>>(D, L, keys, vals);
    launch_radix_sort(keys, vals, d0, s, D.ctr + C_MOVE_LIMIT, st, D.load + L, 1);
    k_keys_dests<<<grid_for(d1), 256, 0, st>>>(D, L, keys2, vals2);
    launch_radix_sort(keys2, vals2, d1, s, D.ctr + C_MOVE_LIMIT, st, D.load + L + 1, 8);
    k_match<<<gs, 256, 0, st>>>(D, vals, vals2);
    k_commit_moves<<<gs, 256, 0, st>>>(D, L, vals, vals2);
  }
  for (int L = D.g.levels - 2; L >= 0; L--)
    if (!level_full(D.g, L)) k_apply_moves<<<gs, 256, 0, st>>>(D, L, keys);
  // refineSubblocks
  k_rescore<<<gs, 256, 0, st>>>(D, keys);
  uint8_t *sel = reinterpret_cast<uint8_t *>(keys2);  // 8*B bytes, reused as selection flags
  for (int L = 1; L < D.g.levels; L++) {
    if (level_full(D.g, L - 1)) continue;  // no free block at level L-1: no refinement (limit 0)
    const long long n8 = 8 * D.g.budget[L];
    const long long nt = (n8 + CMP_TILE - 1) / CMP_TILE;
    k_refine_setup<<<1, 1, 0, st>>>(D, L);
    k_cmp_count<<<(unsigned)nt, 256, 0, st>>>(D, L, nullptr, s.tile_sums);
    k_cmp_scan<<<1, 1024, 0, st>>>(D, s.tile_sums, nt, 1);
    k_cmp_scatter<<<(unsigned)nt, 256, 0, st>>>(D, L, nullptr, s.tile_sums, vals);
    if (D.g.ref_compat) {
      k_record_refines<<<gs, 256, 0, st>>>(D, L, vals, 1);
    } else {
      k_keys_cands<<<gs, 256, 0, st>>>(D, vals, keys, vals2, n8);
      launch_radix_sort(keys, vals2, n8, s, D.ctr + C_SELECT, st, D.ctr + C_NCAND, 1);
      cudaMemsetAsync(sel, 0, (size_t)8 * D.g.B, st);
      k_mark_selected<<<gs, 256, 0, st>>>(D, vals2, sel);
      k_cmp_count<<<(unsigned)nt, 256, 0, st>>>(D, L, sel, s.tile_sums);
      k_cmp_scan<<<1, 1024, 0, st>>>(D, s.tile_sums, nt, 0);
      k_cmp_scatter<<<(unsigned)nt, 256, 0, st>>>(D, L, sel, s.tile_sums, vals);
      k_record_refines<<<gs, 256, 0, st>>>(D, L, vals, 0);
    }
  }
  k_apply_refines<<<gs, 256, 0, st>>>(D);
  k_finish_refines<<<1, 1, 0, st>>>(D);
  // neighbour tables (the refresh after an adaptation) + value propagation for touched blocks
  k_refresh_nbr<<<grid_for(D.g.B * 27), 256, 0, st>>>(D);
  for (int L = D.g.levels - 2; L >= 0; L--) k_propagate<<<gs, 256, 0, st>>>(D, L);
}

// Field-criterion scores one warp per block (used for every simulation whose
// refine criterion is the field one): lanes 0-5 resolve the block's faces,
// the products w*v0, w*v1, w*v2 and the density of the block and its face
// halo go through shared tiles, then each lane computes field_cell_score's
// arithmetic for its two cells from the tiles and the four lanes of a
// subblock reduce the maximum.
__device__ __forceinline__ float2 q_ld2(const Dev &D, size_t own, int lane) {
  if (D.g.mixed) {
    const uint32_t u = reinterpret_cast<const uint32_t *>(D.qh[0] + own)[lane];
    return make_float2(h16_to_f((uint16_t)(u & 0xFFFFu), D.g.mixed), h16_to_f((uint16_t)(u >> 16), D.g.mixed));
  }
  return reinterpret_cast<const float2 *>(D.q[0] + own)[lane];
}
struct StagedScoreOut {
  float ox, oy, oz, gx, gy, gz;
};
__device__ __forceinline__ float field_score_of(const Dev &D, float alpha, float wv2U, float wv2D, float wv1F,
                                                float wv1B, float wv0F, float wv0B, float wv2R, float wv2L,
                                                float wv1R, float wv1L, float wv0U, float wv0D, float qR, float qL,
                                                float qU, float qD, float qF, float qB) {
  const float ox = alpha * ((wv2U - wv2D) - (wv1F - wv1B));
  const float oy = alpha * ((wv0F - wv0B) - (wv2R - wv2L));
  const float oz = alpha * ((wv1R - wv1L) - (wv0U - wv0D));
  const float gxr = alpha * (qR - qL);
  const float gyr = alpha * (qU - qD);
  const float gzr = alpha * (qF - qB);
  const float om = sqrtf(ox * ox + oy * oy + oz * oz);
  const float gr = sqrtf(gxr * gxr + gyr * gyr + gzr * gzr);
  const float a = om / D.ph.vort_t, bb = gr / D.ph.grad_t;
  return fmaxf(0.f, a < bb ? bb : a);
}
struct ScoreBatchP {
  int n, pad;
  long long end[BMAX];  // cumulative block counts (0 for members without the field criterion)
  Dev d[BMAX];
};
// The warps walk the allocated blocks only (each level's allocated blocks are
// the prefix [off, off + load) of its budget range), segment by segment
// (member, level) as k_cells_staged does; a level that level_blocked refuses
// gets the blocked score without loading anything, and the unallocated tails
// of the budget ranges (and the blocks past them) get it from coalesced
// stores after the walk. Results equal scores_fields_body.
__global__ void __launch_bounds__(256) k_scores_staged(const __grid_constant__ ScoreBatchP P) {
  constexpr int W = 8, SX = DCG_TILE_SX, SY = DCG_TILE_SY, TILE = 5 * SX + 5 * SY + 8;
  __shared__ __align__(16) float s_tile[W][4][TILE];
  __shared__ long long s_end[BMAX * MAXL], s_tail[BMAX * MAXL];
  __shared__ uint8_t s_blk[BMAX * MAXL];
  const int nseg = P.n * MAXL;
  for (int i = threadIdx.x; i < nseg; i += blockDim.x) {
    const int mi = i / MAXL, l = i % MAXL;
    const Dev &D = P.d[mi];
    const bool has = l < D.g.levels && P.end[mi] - (mi ? P.end[mi - 1] : 0) > 0;
    const long long ld = has ? __ldcg(D.load + l) : 0;
    s_end[i] = ld;
    // the last level's tail also covers the blocks past every budget range
    const long long past = l == D.g.levels - 1 ? D.g.B - (D.g.off[l] + D.g.budget[l]) : 0;
    s_tail[i] = has ? D.g.budget[l] - ld + past : 0;
    s_blk[i] = (uint8_t)(has && level_blocked(D, l));
    if (blockIdx.x == 0 && l == 0 && has) D.ss[8 * D.g.B] = 0.f;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 1; i < nseg; i++) {
      s_end[i] += s_end[i - 1];
      s_tail[i] += s_tail[i - 1];
    }
  __syncthreads();
  const long long total = s_end[nseg - 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int oA;
  uint32_t hpk[3], hax[3];
  halo_slots<SX, SY>(lane, oA, hpk, hax);
  const unsigned full = 0xffffffffu;
  int seg = 0;
  for (long long t = (long long)blockIdx.x * W + w; t < total; t += (long long)gridDim.x * W) {
    while (t >= s_end[seg]) seg++;
    const Dev &D = P.d[seg / MAXL];
    const uint32_t b = (uint32_t)(D.g.off[seg % MAXL] + (t - (seg ? s_end[seg - 1] : 0)));
    const uint32_t sb = 8u * b + (uint32_t)(lane >> 2);
    if (s_blk[seg]) {  // warp-uniform
      if ((lane & 3) == 0) D.ss[sb] = -FLT_MAX;
      continue;
    }
    const int4 bp = D.pos[b];
    const bool blocked = D.child[sb] != NONE;
    const size_t own = (size_t)b * BV;
    uint32_t e = OUT;
    if (lane < 6) e = D.nbr[27u * b + (lane == 0 ? 4 : lane == 1 ? 22 : lane == 2 ? 10 : lane == 3 ? 16 : lane == 4 ? 12 : 14)];
    size_t hc[3];
#pragma unroll
    for (int q = 0; q < 3; q++) hc[q] = halo_cell(D, b, bp, __shfl_sync(full, e, (int)(hax[q] >> 12)), hpk[q], hax[q]);
    float *T0 = s_tile[w][0], *T1 = s_tile[w][1], *T2 = s_tile[w][2], *TQ = s_tile[w][3];
    const float2 w2 = reinterpret_cast<const float2 *>(D.w + own)[lane];
    const float2 v0 = reinterpret_cast<const float2 *>(D.v[0] + own)[lane];
    const float2 v1 = reinterpret_cast<const float2 *>(D.v[1] + own)[lane];
    const float2 v2 = reinterpret_cast<const float2 *>(D.v[2] + own)[lane];
    const float2 q2 = q_ld2(D, own, lane);
    const float2 p0 = make_float2(w2.x * v0.x, w2.y * v0.y), p1 = make_float2(w2.x * v1.x, w2.y * v1.y),
                 p2 = make_float2(w2.x * v2.x, w2.y * v2.y);
    *reinterpret_cast<float2 *>(T0 + oA) = p0;
    *reinterpret_cast<float2 *>(T1 + oA) = p1;
    *reinterpret_cast<float2 *>(T2 + oA) = p2;
    *reinterpret_cast<float2 *>(TQ + oA) = q2;
#pragma unroll
    for (int q = 0; q < 3; q++) {  // slot q lies on the faces of axis q
      const size_t c = hc[q];
      const float hw = D.w[c];
      const uint32_t at = hpk[q] & 511u;
      if (q != 0) T0[at] = hw * D.v[0][c];
      if (q != 1) T1[at] = hw * D.v[1][c];
      if (q != 2) T2[at] = hw * D.v[2][c];
      TQ[at] = q_ld(D, 0, c);
    }
    __syncwarp();
    const int scale = 1 << bp.w;
    const float alpha = 0.5f * D.ph.rdx / (float)scale;
    const float2 w0U = *reinterpret_cast<const float2 *>(T0 + oA + SY), w0D = *reinterpret_cast<const float2 *>(T0 + oA - SY);
    const float2 w1R = *reinterpret_cast<const float2 *>(T1 + oA + SX), w1L = *reinterpret_cast<const float2 *>(T1 + oA - SX);
    const float2 w2U = *reinterpret_cast<const float2 *>(T2 + oA + SY), w2D = *reinterpret_cast<const float2 *>(T2 + oA - SY);
    const float2 w2R = *reinterpret_cast<const float2 *>(T2 + oA + SX), w2L = *reinterpret_cast<const float2 *>(T2 + oA - SX);
    const float2 qR = *reinterpret_cast<const float2 *>(TQ + oA + SX), qL = *reinterpret_cast<const float2 *>(TQ + oA - SX);
    const float2 qU = *reinterpret_cast<const float2 *>(TQ + oA + SY), qD = *reinterpret_cast<const float2 *>(TQ + oA - SY);
    const float w0B = T0[oA - 1], w0F = T0[oA + 2], w1B = T1[oA - 1], w1F = T1[oA + 2], qB = TQ[oA - 1],
                qF = TQ[oA + 2];
    __syncwarp();
    // cell A (z even): +z neighbour is cell B; cell B: -z neighbour is cell A
    const float mA = field_score_of(D, alpha, w2U.x, w2D.x, p1.y, w1B, p0.y, w0B, w2R.x, w2L.x, w1R.x, w1L.x, w0U.x,
                                    w0D.x, qR.x, qL.x, qU.x, qD.x, q2.y, qB);
    const float mB = field_score_of(D, alpha, w2U.y, w2D.y, w1F, p1.x, w0F, p0.x, w2R.y, w2L.y, w1R.y, w1L.y, w0U.y,
                                    w0D.y, qR.y, qL.y, qU.y, qD.y, qF, q2.x);
    float mm = blocked ? 0.f : fmaxf(mA, mB);
    mm = fmaxf(mm, __shfl_xor_sync(full, mm, 1));
    mm = fmaxf(mm, __shfl_xor_sync(full, mm, 2));
    if ((lane & 3) == 0) D.ss[sb] = blocked ? -FLT_MAX : mm;
  }
  // the unallocated tails: 8 subblock scores per block, float4 stores
  const long long ttot = s_tail[nseg - 1];
  seg = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * ttot;
       i += (long long)gridDim.x * blockDim.x) {
    const long long tb = i >> 1;  // tail block
    while (tb >= s_tail[seg]) seg++;
    const Dev &D = P.d[seg / MAXL];
    const int l = seg % MAXL;
    const long long b = D.g.off[l] + (s_end[seg] - (seg ? s_end[seg - 1] : 0)) + (tb - (seg ? s_tail[seg - 1] : 0));
    reinterpret_cast<float4 *>(D.ss + 8 * b)[i & 1] = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX);
  }
}
static unsigned scores_staged_grid() {
  static unsigned g = 0;
  if (!g) {
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_scores_staged, 256, 0);
    g = (unsigned)(sms * (occ > 0 ? occ : 1));
  }
  return g;
}
// field-criterion scores of the members with that criterion (in one launch)
static void launch_scores_staged(const Dev *d, int n, cudaStream_t st) {
  ScoreBatchP P{};
  P.n = n;
  long long e = 0;
  for (int i = 0; i < n; i++) {
    P.d[i] = d[i];
    if (d[i].ph.criterion != 0) e += d[i].g.B;
    P.end[i] = e;
  }
  if (e > 0) k_scores_staged<<<scores_staged_grid(), 256, 0, st>>>(P);
}

// ------------------------------------------------------- batched adaptation
// launch_adapt's sequence for up to BMAX members, one launch per adaptation
// kernel: a CTA picks its member from the cumulative CTA counts and runs the
// single-simulation body with its member-local CTA index and grid size. A
// member without the launch's level (or of the other selection mode) gets no
// CTAs. The bodies are the single simulation's, so the results are too.
enum : int {
  A_CLEAR, A_SCORES, A_BLOCK_SCORES, A_MOVE_SETUP, A_KEYS, A_MATCH, A_COMMIT, A_APPLY_MOVES, A_REFINE_SETUP,
  A_CMP_COUNT, A_CMP_SCAN, A_CMP_SCATTER, A_RECORD, A_KEYS_CANDS, A_CLEAR_SEL, A_MARK, A_APPLY_REFINES,
  A_FINISH, A_NBR, A_PROPAGATE, A_RESCORE
};
struct AdaptBatchP {
  int n, L;
  long long end[BMAX];
  uint32_t *p0[BMAX], *p1[BMAX], *p2[BMAX], *p3[BMAX];  // per-op buffers
  long long nn[BMAX];
  int arg[BMAX];
  Dev d[BMAX];
};
static_assert(sizeof(AdaptBatchP) < 32000, "kernel parameter space");

// clears the counters and the block flags of one member
__device__ __forceinline__ void clear_body(const Dev &D, unsigned bx, unsigned gx) {
  const long long n = D.g.B > C_COUNT ? D.g.B : C_COUNT;
  for (long long i = (long long)bx * blockDim.x + threadIdx.x; i < n; i += (long long)gx * blockDim.x) {
    if (i < C_COUNT) D.ctr[i] = 0;
    if (i < D.g.B) D.flags[i] = 0;
  }
}

template <int OP, int T> __global__ void __launch_bounds__(T) k_adapt_batch(const __grid_constant__ AdaptBatchP P) {
  int s = 0;
  while (s < P.n - 1 && blockIdx.x >= P.end[s]) s++;
  const long long first = s ? P.end[s - 1] : 0;
  const unsigned bx = (unsigned)(blockIdx.x - first), gx = (unsigned)(P.end[s] - first);
  const Dev &D = P.d[s];
  const int L = P.L;
  if constexpr (OP == A_CLEAR) clear_body(D, bx, gx);
  if constexpr (OP == A_SCORES) {
    if (D.ph.criterion == 0)
      scores_geo_body(D, bx, gx);
    else
      scores_fields_body(D, bx, gx);
  }
  if constexpr (OP == A_BLOCK_SCORES) block_scores_body(D, bx, gx);
  if constexpr (OP == A_MOVE_SETUP) {
    if (threadIdx.x == 0) move_setup_body(D, L, bx, gx);
  }
  if constexpr (OP == A_KEYS) {  // block keys of level L and destination keys of level L+1
    const long long nb = (P.nn[s] + T - 1) / T;
    if (bx < nb)
      keys_blocks_body(D, L, P.p0[s], P.p1[s], bx, (unsigned)nb);
    else
      keys_dests_body(D, L, P.p2[s], P.p3[s], bx - (unsigned)nb, gx - (unsigned)nb);
  }
  if constexpr (OP == A_MATCH) match_body(D, P.p0[s], P.p1[s], bx, gx);
  if constexpr (OP == A_COMMIT) commit_moves_body(D, L, P.p0[s], P.p1[s], bx, gx);
  if constexpr (OP == A_APPLY_MOVES) apply_moves_body(D, L, P.p0[s], bx, gx);
  if constexpr (OP == A_RESCORE) rescore_body(D, P.p0[s], bx, gx);
  if constexpr (OP == A_REFINE_SETUP) {
    if (threadIdx.x == 0) refine_setup_body(D, L, bx, gx);
  }
  if constexpr (OP == A_CMP_COUNT)
    cmp_count_body(D, L, reinterpret_cast<const uint8_t *>(P.p0[s]), P.p1[s], bx, gx);
  if constexpr (OP == A_CMP_SCAN) cmp_scan_body(D, P.p1[s], P.nn[s], P.arg[s], bx, gx);
  if constexpr (OP == A_CMP_SCATTER)
    cmp_scatter_body(D, L, reinterpret_cast<const uint8_t *>(P.p0[s]), P.p1[s], P.p2[s], bx, gx);
  if constexpr (OP == A_RECORD) record_refines_body(D, L, P.p0[s], P.arg[s], bx, gx);
  if constexpr (OP == A_KEYS_CANDS) keys_cands_body(D, P.p0[s], P.p1[s], P.p2[s], P.nn[s], bx, gx);
  if constexpr (OP == A_CLEAR_SEL) {
    if (D.ctr[C_SELECT] == 0) return;  // no selection at this level
    uint32_t *w = P.p0[s];
    for (long long i = (long long)bx * T + threadIdx.x; i < P.nn[s]; i += (long long)gx * T) w[i] = 0;
  }
  if constexpr (OP == A_MARK) mark_selected_body(D, P.p0[s], reinterpret_cast<uint8_t *>(P.p1[s]), bx, gx);
  if constexpr (OP == A_APPLY_REFINES) apply_refines_body(D, bx, gx);
  if constexpr (OP == A_FINISH) {
    if (threadIdx.x == 0) finish_refines_body(D, bx, gx);
  }
  if constexpr (OP == A_NBR) refresh_nbr_body(D, bx, gx);
  if constexpr (OP == A_PROPAGATE) propagate_body(D, L, bx, gx);
}

namespace {
struct AdaptLauncher {
  const AdaptMember *m;
  int n;
  unsigned gs;  // grid-stride CTAs per member
  cudaStream_t st;
  void sort(const SortSeg *seg, int ns) { launch_radix_sort_batch(seg, ns, st); }
  AdaptBatchP P{};

  AdaptLauncher(const AdaptMember *mm, int nn, int sms, cudaStream_t s) : m(mm), n(nn), st(s) {
    P.n = n;
    for (int i = 0; i < n; i++) P.d[i] = m[i].D;
    const int total = sms > 0 ? sms * 4 : 512;
    gs = (unsigned)std::max(32, (total + n - 1) / n);
  }
  // CTA counts from ctas(i) (0 = member i sits the launch out); false when no CTA runs
  template <typename F> bool counts(F ctas) {
    long long e = 0;
    for (int i = 0; i < n; i++) {
      e += ctas(i);
      P.end[i] = e;
    }
    return e > 0;
  }
  template <int OP, int T = 256, typename F> void go(F ctas) {
    if (counts(ctas)) k_adapt_batch<OP, T><<<(unsigned)P.end[n - 1], T, 0, st>>>(P);
  }
  int levels(int i) const { return m[i].D.g.levels; }
  long long B(int i) const { return m[i].D.g.B; }

  void scores() {
    go<A_SCORES>([&](int i) { return m[i].D.ph.criterion == 0 ? (long long)grid_for(8 * B(i) + 1) : 0ll; });
    Dev d[BMAX];
    for (int i = 0; i < n; i++) d[i] = m[i].D;
    launch_scores_staged(d, n, st);
  }
  // compaction of level L's flagged subblocks (sel null: threshold test) into p2
  void compact(int L, bool sel, const std::vector<bool> &in) {
    auto nt = [&](int i) { return (8 * m[i].D.g.budget[L] + CMP_TILE - 1) / CMP_TILE; };
    for (int i = 0; i < n; i++) {
      P.p0[i] = sel ? m[i].keys2 : nullptr;
      P.p1[i] = m[i].S.tile_sums;
      P.p2[i] = m[i].vals;
      P.nn[i] = nt(i);
      P.arg[i] = sel ? 0 : 1;  // the threshold compaction decides C_SELECT
    }
    go<A_CMP_COUNT>([&](int i) { return in[i] ? nt(i) : 0; });
    go<A_CMP_SCAN, 1024>([&](int i) { return in[i] ? 1 : 0; });
    go<A_CMP_SCATTER>([&](int i) { return in[i] ? nt(i) : 0; });
  }

  void run() {
    int maxl = 0;
    for (int i = 0; i < n; i++) maxl = std::max(maxl, levels(i));
    go<A_CLEAR>([&](int i) { return (long long)std::min<long long>(gs, grid_for(std::max<long long>(B(i), C_COUNT))); });
    // moveBlocks
    scores();
    go<A_BLOCK_SCORES>([&](int i) { return (long long)grid_for(B(i)); });
    for (int L = 0; L < maxl - 1; L++) {
      P.L = L;
      auto has = [&](int i) { return L < levels(i) - 1 && !level_full(m[i].D.g, L); };
      go<A_MOVE_SETUP, 32>([&](int i) { return has(i) ? 1 : 0; });
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].keys;
        P.p1[i] = m[i].vals;
        P.p2[i] = m[i].keys2;
        P.p3[i] = m[i].vals2;
        P.nn[i] = m[i].D.g.budget[L];
      }
      go<A_KEYS>([&](int i) {
        return has(i) ? (long long)grid_for(m[i].D.g.budget[L]) + grid_for(8 * m[i].D.g.budget[L + 1]) : 0;
      });
      SortSeg seg[SORT_SEGS];
      int ns = 0;
      for (int i = 0; i < n; i++) {
        if (!has(i)) continue;
        const long long *act = m[i].D.ctr + C_MOVE_LIMIT;
        // allocated prefixes only: the unallocated tails already sit in their
        // stable-sorted place (largest keys, index order)
        seg[ns++] = SortSeg{m[i].keys, m[i].vals, m[i].D.g.budget[L], act, m[i].S2, m[i].D.load + L, 1};
        seg[ns++] = SortSeg{m[i].keys2, m[i].vals2, 8 * m[i].D.g.budget[L + 1], act, m[i].S, m[i].D.load + L + 1, 8};
      }
      sort(seg, ns);
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].vals;
        P.p1[i] = m[i].vals2;
      }
      go<A_MATCH>([&](int i) { return has(i) ? gs : 0u; });
      go<A_COMMIT>([&](int i) { return has(i) ? gs : 0u; });
    }
    for (int i = 0; i < n; i++) P.p0[i] = m[i].keys;  // previous parents of the moved blocks
    for (int L = maxl - 2; L >= 0; L--) {
      P.L = L;
      go<A_APPLY_MOVES>([&](int i) { return L < levels(i) - 1 && !level_full(m[i].D.g, L) ? gs : 0u; });
    }
    // refineSubblocks
    go<A_RESCORE>([&](int i) { return gs; });
    for (int L = 1; L < maxl; L++) {
      P.L = L;
      std::vector<bool> in(n), compat(n), score(n);
      for (int i = 0; i < n; i++) {
        in[i] = L < levels(i) && !level_full(m[i].D.g, L - 1);
        compat[i] = in[i] && m[i].D.g.ref_compat;
        score[i] = in[i] && !m[i].D.g.ref_compat;
      }
      go<A_REFINE_SETUP, 32>([&](int i) { return in[i] ? 1 : 0; });
      compact(L, false, in);
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].vals;
        P.arg[i] = 1;
      }
      go<A_RECORD>([&](int i) { return compat[i] ? gs : 0u; });
      if (std::none_of(score.begin(), score.end(), [](bool b) { return b; })) continue;
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].vals;
        P.p1[i] = m[i].keys;
        P.p2[i] = m[i].vals2;
        P.nn[i] = 8 * m[i].D.g.budget[L];
      }
      go<A_KEYS_CANDS>([&](int i) { return score[i] ? gs : 0u; });
      SortSeg seg[SORT_SEGS];
      int ns = 0;
      for (int i = 0; i < n; i++)
        if (score[i])
          seg[ns++] = SortSeg{m[i].keys, m[i].vals2, 8 * m[i].D.g.budget[L], m[i].D.ctr + C_SELECT, m[i].S,
                              m[i].D.ctr + C_NCAND, 1};  // the compacted candidates only, when selecting
      sort(seg, ns);
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].keys2;
        P.nn[i] = 2 * B(i);  // 8*B selection bytes as words
      }
      go<A_CLEAR_SEL>([&](int i) { return score[i] ? gs : 0u; });
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].vals2;
        P.p1[i] = m[i].keys2;
      }
      go<A_MARK>([&](int i) { return score[i] ? gs : 0u; });
      compact(L, true, score);
      for (int i = 0; i < n; i++) {
        P.p0[i] = m[i].vals;
        P.arg[i] = 0;
      }
      go<A_RECORD>([&](int i) { return score[i] ? gs : 0u; });
    }
    go<A_APPLY_REFINES>([&](int i) { return gs; });
    go<A_FINISH, 32>([&](int i) { return 1; });
    // neighbour tables + value propagation for touched blocks
    go<A_NBR>([&](int i) { return (long long)grid_for(B(i) * 27); });
    for (int L = maxl - 2; L >= 0; L--) {
      P.L = L;
      go<A_PROPAGATE>([&](int i) { return L < levels(i) - 1 ? gs : 0u; });
    }
  }
};
}  // namespace

void launch_adapt_batch(const AdaptMember *m, int n, int sms, cudaStream_t st) {
  if (n <= 0 || n > BMAX) return;
  AdaptLauncher(m, n, sms, st).run();
}

// ------------------------------------------------------------------ stats
// k_dcgrid_debug_stats (dcgrid_structure.cu:224-251) plus mass and leaf
// counts; warp-shuffle reductions, one double atomic per warp.
__global__ void __launch_bounds__(256) k_stats(Dev D) {
  stats_cell(D, (long long)blockIdx.x * 4 + (threadIdx.x >> 6), threadIdx.x & 63);
}
void launch_stats(const Dev &D, cudaStream_t st) {
  cudaMemsetAsync(D.red, 0, sizeof(double) * 32, st);
  k_stats<<<(unsigned)((D.g.B + 3) / 4), 256, 0, st>>>(D);
}

// Dense resampling: every finest cell takes the leaf value that covers it.
// `mode` is the storage format of src (0 FP32, 1 BF16, 2 FP16).
__global__ void __launch_bounds__(256) k_to_dense(Dev D, const void *src, int mode, float *dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)D.g.gx * D.g.gy * D.g.gz;
  if (i >= n) return;
  const int x = (int)(i % D.g.gx), y = (int)((i / D.g.gx) % D.g.gy), z = (int)(i / ((long long)D.g.gx * D.g.gy));
  int lev;
  const uint32_t b = locate(D, x, y, z, 0, lev);
  const int4 bp = D.pos[b];
  const size_t c = (size_t)b * BV + local_of((x >> lev) - bp.x, (y >> lev) - bp.y, (z >> lev) - bp.z);
  dst[i] = mode ? h16_to_f(static_cast<const uint16_t *>(src)[c], mode) : static_cast<const float *>(src)[c];
}
void launch_fields_to_dense(const Dev &D, const void *src, int mode, float *dst, cudaStream_t st) {
  const long long n = (long long)D.g.gx * D.g.gy * D.g.gz;
  k_to_dense<<<grid_for(n), 256, 0, st>>>(D, src, mode, dst);
}

// Conversions between FP32 and 16-bit scalar storage (field access).
__global__ void __launch_bounds__(256) k_h16_to_f32(const uint16_t *src, float *dst, long long n, int mode) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = h16_to_f(src[i], mode);
}
__global__ void __launch_bounds__(256) k_f32_to_h16(const float *src, uint16_t *dst, long long n, int mode) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = f_to_h16(src[i], mode);
}
void launch_h16_to_f32(const uint16_t *src, float *dst, long long n, int mode, cudaStream_t st) {
  k_h16_to_f32<<<grid_for(n), 256, 0, st>>>(src, dst, n, mode);
}
void launch_f32_to_h16(const float *src, uint16_t *dst, long long n, int mode, cudaStream_t st) {
  k_f32_to_h16<<<grid_for(n), 256, 0, st>>>(src, dst, n, mode);
}

// The reference-format 216-entry apron table, derived from neighbour tables.
__global__ void __launch_bounds__(216) k_apron_table(Dev D, long long *dst) {
  const long long b = blockIdx.x;
  const int a = threadIdx.x;
  const int4 bp = D.pos[b];
  if (bp.w < 0) {
    dst[b * 216 + a] = -1;
    return;
  }
  dst[b * 216 + a] = (long long)apron_cell(D, (uint32_t)b, bp, a / 36, (a / 6) % 6, a % 6);
}
void launch_apron_table(const Dev &D, long long *dst, cudaStream_t st) {
  k_apron_table<<<(unsigned)D.g.B, 216, 0, st>>>(D, dst);
}

}  // namespace dcg
