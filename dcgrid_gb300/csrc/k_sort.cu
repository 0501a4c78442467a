// k_sort.cu — stable LSD radix sort of (u32 key, u32 value) pairs, used to
// rank adaptation candidates on the device (replaces the host-side
// std::nth_element / std::sort of fluid_simulation_dcgrid.cu:387-408).
//
// Four 8-bit passes; each pass: tile histograms -> per-digit column scans ->
// digit bases -> stable scatter. The scatter ranks equal digits with
// __match_any_sync inside a warp and a per-digit running offset across warps
// and rounds, so the order of equal keys is preserved (ties stay in index
// order, which the selection relies on).
#include <utility>

#include "dcg_kernels.h"

namespace dcg {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

long long sort_tiles(long long n) { return (n + RS_TILE - 1) / RS_TILE; }

__device__ inline bool gate_off(const long long *active) { return active && *active == 0; }
// entries to sort: n, or the device-side prefix min(n, nmul * *ndev)
__device__ inline long long eff_n(long long n, const long long *ndev, int nmul) {
  if (!ndev) return n;
  const long long m = (long long)nmul * *ndev;
  return m < n ? m : n;
}

__device__ __forceinline__ void rs_hist_body(const uint32_t *__restrict__ keys, long long n, int shift, uint32_t *__restrict__ hist, long long ntiles, const long long *active, unsigned bx, unsigned gx) {
  if (gate_off(active)) return;
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)bx * RS_TILE;
  for (int r = 0; r < RS_ITEMS; r++) {
    const long long i = base + r * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[(__ldcg(keys + i) >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * ntiles + bx] = h[threadIdx.x];
}
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t *__restrict__ keys, long long n, int shift, uint32_t *__restrict__ hist, long long ntiles, const long long *active, const long long *ndev, int nmul) { rs_hist_body(keys, eff_n(n, ndev, nmul), shift, hist, ntiles, active, blockIdx.x, gridDim.x); }

// Block-wide exclusive scan of one value per thread (256 threads); returns
// the exclusive prefix and writes the block total to *total.
__device__ inline uint32_t block_exclusive_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t warp_sums[RS_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < RS_THREADS / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < RS_THREADS / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const uint32_t before = warp == 0 ? 0 : warp_sums[warp - 1];
  *total = warp_sums[RS_THREADS / 32 - 1];
  __syncthreads();
  return before + x - v;
}

// One CTA per digit: exclusive scan of that digit's tile counts, in place.
__device__ __forceinline__ void rs_scan_cols_body(uint32_t *__restrict__ hist, long long ntiles, uint32_t *__restrict__ totals, const long long *active, unsigned bx, unsigned gx) {
  if (gate_off(active)) return;
  uint32_t *col = hist + (long long)bx * ntiles;
  uint32_t carry = 0;
  for (long long t0 = 0; t0 < ntiles; t0 += RS_THREADS) {
    const long long t = t0 + threadIdx.x;
    const uint32_t v = t < ntiles ? __ldcg(col + t) : 0;
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan(v, &tot);
    if (t < ntiles) col[t] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) totals[bx] = carry;
}
__global__ void __launch_bounds__(RS_THREADS) k_rs_scan_cols(uint32_t *__restrict__ hist, long long ntiles, uint32_t *__restrict__ totals, const long long *active) { rs_scan_cols_body(hist, ntiles, totals, active, blockIdx.x, gridDim.x); }

__device__ __forceinline__ void rs_scan_totals_body(uint32_t *__restrict__ totals, const long long *active, unsigned bx, unsigned gx) {
  if (gate_off(active)) return;
  uint32_t tot;
  const uint32_t v = __ldcg(totals + threadIdx.x);
  const uint32_t ex = block_exclusive_scan(v, &tot);
  totals[threadIdx.x] = ex;
}
__global__ void __launch_bounds__(RS_THREADS) k_rs_scan_totals(uint32_t *__restrict__ totals, const long long *active) { rs_scan_totals_body(totals, active, blockIdx.x, gridDim.x); }

__device__ __forceinline__ void rs_scatter_body(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, long long n, int shift, const uint32_t *__restrict__ hist, const uint32_t *__restrict__ totals, long long ntiles, const long long *active, unsigned bx, unsigned gx) {
  if (gate_off(active)) return;
  __shared__ uint32_t s_base[256];
  __shared__ uint32_t s_wcnt[RS_THREADS / 32][256];
  __shared__ uint32_t s_round[256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = threadIdx.x;
  s_base[t] = __ldcg(totals + t) + __ldcg(hist + (long long)t * ntiles + bx);
  const long long base = (long long)bx * RS_TILE;
  for (int r = 0; r < RS_ITEMS; r++) {
    const long long i = base + r * RS_THREADS + t;
    const bool valid = i < n;
    const uint32_t k = valid ? __ldcg(kin + i) : 0u;
    const uint32_t d = valid ? ((k >> shift) & 255u) : (256u + lane);
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; w++) s_wcnt[w][t] = 0;
    __syncthreads();
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (valid && lane == __ffs(peers) - 1) s_wcnt[warp][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < RS_THREADS / 32; w++) {
        const uint32_t c = s_wcnt[w][t];
        s_wcnt[w][t] = run;
        run += c;
      }
      s_round[t] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_base[d] + s_wcnt[warp][d] + (uint32_t)rank;
      kout[pos] = k;
      vout[pos] = __ldcg(vin + i);
    }
    __syncthreads();
    s_base[t] += s_round[t];
    __syncthreads();
  }
}
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, long long n, int shift, const uint32_t *__restrict__ hist, const uint32_t *__restrict__ totals, long long ntiles, const long long *active, const long long *ndev, int nmul) { rs_scatter_body(kin, vin, kout, vout, eff_n(n, ndev, nmul), shift, hist, totals, ntiles, active, blockIdx.x, gridDim.x); }

void launch_radix_sort(uint32_t *keys, uint32_t *vals, long long n, const SortScratch &s,
                       const long long *active, cudaStream_t st, const long long *ndev, int nmul) {
  if (n <= 0) return;
  const long long nt = sort_tiles(n);
  uint32_t *kin = keys, *vin = vals, *kout = s.k1, *vout = s.v1;
  for (int pass = 0; pass < 4; pass++) {
    const int shift = 8 * pass;
    k_rs_hist<<<(unsigned)nt, RS_THREADS, 0, st>>>(kin, n, shift, s.hist, nt, active, ndev, nmul);
    k_rs_scan_cols<<<256, RS_THREADS, 0, st>>>(s.hist, nt, s.totals, active);
    k_rs_scan_totals<<<1, RS_THREADS, 0, st>>>(s.totals, active);
    k_rs_scatter<<<(unsigned)nt, RS_THREADS, 0, st>>>(kin, vin, kout, vout, n, shift, s.hist,
                                                     s.totals, nt, active, ndev, nmul);
    uint32_t *tk = kin, *tv = vin;
    kin = kout; vin = vout;
    kout = tk; vout = tv;
  }
  // four passes: the result is back in (keys, vals)
}

// ---- batched sorts: segments (one or two per member) sorted by the same
// launches; a CTA picks its segment from the cumulative CTA counts.
struct SortBatchP {
  int nseg, shift;
  long long end[SORT_SEGS];
  const uint32_t *kin[SORT_SEGS], *vin[SORT_SEGS];
  uint32_t *kout[SORT_SEGS], *vout[SORT_SEGS];
  uint32_t *hist[SORT_SEGS], *totals[SORT_SEGS];
  const long long *active[SORT_SEGS];
  long long n[SORT_SEGS], nt[SORT_SEGS];
  const long long *ndev[SORT_SEGS];
  int nmul[SORT_SEGS];
};

template <int OP> __global__ void __launch_bounds__(RS_THREADS) k_rs_batch(const __grid_constant__ SortBatchP P) {
  int s = 0;
  while (s < P.nseg - 1 && blockIdx.x >= P.end[s]) s++;
  const long long first = s ? P.end[s - 1] : 0;
  const unsigned bx = (unsigned)(blockIdx.x - first), gx = (unsigned)(P.end[s] - first);
  if constexpr (OP == 0)
    rs_hist_body(P.kin[s], eff_n(P.n[s], P.ndev[s], P.nmul[s]), P.shift, P.hist[s], P.nt[s], P.active[s], bx, gx);
  if constexpr (OP == 1) rs_scan_cols_body(P.hist[s], P.nt[s], P.totals[s], P.active[s], bx, gx);
  if constexpr (OP == 2) rs_scan_totals_body(P.totals[s], P.active[s], bx, gx);
  if constexpr (OP == 3)
    rs_scatter_body(P.kin[s], P.vin[s], P.kout[s], P.vout[s], eff_n(P.n[s], P.ndev[s], P.nmul[s]), P.shift,
                    P.hist[s], P.totals[s], P.nt[s], P.active[s], bx, gx);
}

void launch_radix_sort_batch(const SortSeg *seg, int nseg, cudaStream_t st) {
  SortBatchP P{};
  uint32_t *k[SORT_SEGS], *v[SORT_SEGS], *ko[SORT_SEGS], *vo[SORT_SEGS];
  for (int i = 0; i < nseg; i++) {
    P.n[i] = seg[i].n > 0 ? seg[i].n : 0;
    P.nt[i] = sort_tiles(P.n[i]);
    P.hist[i] = seg[i].s.hist;
    P.totals[i] = seg[i].s.totals;
    P.active[i] = seg[i].active;
    P.ndev[i] = seg[i].ndev;
    P.nmul[i] = seg[i].nmul;
    k[i] = seg[i].keys;
    v[i] = seg[i].vals;
    ko[i] = seg[i].s.k1;
    vo[i] = seg[i].s.v1;
  }
  P.nseg = nseg;
  auto ends = [&](long long per_tile, long long fixed) {
    long long e = 0;
    for (int i = 0; i < nseg; i++) {
      if (P.n[i] > 0) e += per_tile * P.nt[i] + fixed;
      P.end[i] = e;
    }
    return (unsigned)e;
  };
  for (int pass = 0; pass < 4; pass++) {
    P.shift = 8 * pass;
    for (int i = 0; i < nseg; i++) {
      P.kin[i] = k[i];
      P.vin[i] = v[i];
      P.kout[i] = ko[i];
      P.vout[i] = vo[i];
    }
    const unsigned tiles = ends(1, 0);
    if (tiles == 0) return;
    k_rs_batch<0><<<tiles, RS_THREADS, 0, st>>>(P);
    k_rs_batch<1><<<ends(0, 256), RS_THREADS, 0, st>>>(P);
    k_rs_batch<2><<<ends(0, 1), RS_THREADS, 0, st>>>(P);
    k_rs_batch<3><<<ends(1, 0), RS_THREADS, 0, st>>>(P);
    for (int i = 0; i < nseg; i++) {
      std::swap(k[i], ko[i]);
      std::swap(v[i], vo[i]);
    }
  }
}

}  // namespace dcg
