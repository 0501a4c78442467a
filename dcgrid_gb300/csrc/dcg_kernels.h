// dcg_kernels.h — host-side launchers of the device kernels.
#pragma once
#include <cuda_runtime.h>

#include "dcg_dev.cuh"

namespace dcg {

struct FieldList {
  void *f[6];
  int mode[6];  // 0 = FP32, 1 = BF16, 2 = FP16 storage
  int n;
};

// stable LSD radix sort of (key, value) u32 pairs; scratch sized by sort_scratch_words
struct SortScratch {
  uint32_t *k1, *v1;   // ping-pong buffers (n)
  uint32_t *hist;      // 256 * tiles
  uint32_t *totals;    // 256
  uint32_t *tile_sums; // tiles (compaction)
  long long max_n;
};
long long sort_tiles(long long n);
void launch_radix_sort(uint32_t *keys, uint32_t *vals, long long n, const SortScratch &s,
                       const long long *active, cudaStream_t st, const long long *ndev = nullptr, int nmul = 1);
// many sorts in the same launches (at most SORT_SEGS segments, each with its own scratch)
constexpr int SORT_SEGS = 32;
struct SortSeg {
  uint32_t *keys, *vals;
  long long n;
  const long long *active;
  SortScratch s;
  // optional: sort only the first min(n, nmul * *ndev) entries (a device-side
  // count); callers use it where the entries after that prefix are already in
  // their stable-sorted place (equal largest keys in index order) or unused
  const long long *ndev;
  int nmul;
};
void launch_radix_sort_batch(const SortSeg *seg, int nseg, cudaStream_t st);

// k_fluid.cu
void launch_advect_velocity(const Dev &D, cudaStream_t st);
void launch_advect_scalars(const Dev &D, cudaStream_t st);
void launch_sources(const Dev &D, cudaStream_t st);
void launch_add_noise(const Dev &D, unsigned long long seed, float amp, cudaStream_t st);
void launch_restrict(const Dev &D, const FieldList &fl, cudaStream_t st);
void launch_divergence(const Dev &D, cudaStream_t st);
void launch_jacobi(const Dev &D, int level, const float *src, float *dst, cudaStream_t st);
void launch_prolongate(const Dev &D, int level, cudaStream_t st);
void launch_apply_pressure(const Dev &D, cudaStream_t st);
// defect correction: FP64 residual into D.rr (+ norms), p += e
void launch_add_correction(const Dev &D, cudaStream_t st);
// cooperative persistent solve of one level (prolongation + sweeps)
int level_solve_grid(int sms);
void launch_level_solve(const Dev &D, int level, int prolong, int sweeps, int grid, int epoch_sync, cudaStream_t st);

// ---- batched launches (many independent simulations per launch)
// Member devices travel in the kernel parameters (__grid_constant__, read
// through the constant cache); BMAX members fit the 32 KB parameter space.
constexpr int BMAX = 16;
// words of one block's description in a staged cascade sweep (fill_block_info)
constexpr int BI_OWN = 0, BI_ALPHA = 1, BI_CODES = 2, BI_FACE = 4, BI_POS = 10, BI_WORDS = 16;
// cell stages: 0 advect velocity, 1 advect scalars, 2 divergence, 3 apply
// pressure, 4 statistics (into each member's red; zero it first), 5 apply
// pressure and advect scalars in one staged pass (the results of 3 then 1),
// 6 the FP64 defect residual of correction pass `arg` (staged only)
struct CellBatch {
  int n, arg;
  long long end[BMAX];  // cumulative CTA count of members 0..s
  Dev d[BMAX];
};
struct RestrictBatch {
  int n, level;
  long long end[BMAX];
  Dev d[BMAX];
  FieldList fl[BMAX];
};
// Cascade round r solves level maxtop - r of every member that has it (finest
// levels aligned); p and p~ of all members are slices of two arenas.
struct SolveBatch {
  int n, maxtop, prolong, pad;
  float *p, *pt;
  const float *div;  // divergence arena (same layout as p)
  uint32_t *binfo;   // block descriptions of the round's level, BI_WORDS words per level block
  uint32_t *bar, *err;
  unsigned long long arena[BMAX];  // first cell of member s in the arenas
  Dev d[BMAX];
};
static_assert(sizeof(RestrictBatch) < 32000 && sizeof(SolveBatch) < 32000, "kernel parameter space");
// persistent: a grid of a few CTAs per SM over the allocated blocks only
void launch_cells_batch(int stage, CellBatch &P, int tile, cudaStream_t st, bool persistent = false);
void launch_restrict_batch(RestrictBatch &P, cudaStream_t st);
// statistics read-out of a batch: zero the members' reduction slots; copy
// every member's slots, counters, loads and error word into one record array
struct StatRecord {
  double red[32];
  long long ctr[C_COUNT], load[MAXL];
  uint32_t err, pad;
  double dn[4];  // defect correction: ||r||^2, ||div||^2 before the first and after the last pass
};
void launch_stats_zero(const CellBatch &P, cudaStream_t st);
void launch_stats_gather(const CellBatch &P, StatRecord *dst, cudaStream_t st);
// batched defect correction's update p += e (its residual is cell stage 6)
void launch_add_correction_batch(CellBatch &P, cudaStream_t st);
// CTAs of the batched solve for a variant (cache depth 0, 3, 4, 8; 16, 18, 19: pipelined
// staged sweeps with two tile buffers and cache depth 0, 2, 3; 32, 34, 35: three buffers;
// 64, 66: two buffers, registers for 5 CTAs per SM)
// and CTAs per SM (0 = occupancy limit)
int batch_solve_grid(int sms, int cache, int ctas_per_sm);
bool solve_variant_valid(int cache);
void launch_level_solve_batch(const SolveBatch &P, int round, int sweeps, int grid, int cache, int tree,
                              cudaStream_t st);

// self-check of the solver's division by six: bad[0] += mismatches, bad[1] = min mismatching input
void launch_check_div6(unsigned long long *bad, int sms, cudaStream_t st);
int launch_barrier_probe(uint32_t *bar, uint32_t *errw, unsigned limit, unsigned nctas, cudaStream_t st);

// k_topology.cu
void launch_init_blocks(const Dev &D, cudaStream_t st);
void launch_activate_level(const Dev &D, int level, cudaStream_t st);
void launch_build_nbr(const Dev &D, bool only_if_touched, cudaStream_t st);
void launch_adapt(const Dev &D, const SortScratch &s, uint32_t *keys, uint32_t *vals,
                  uint32_t *keys2, uint32_t *vals2, int sms, cudaStream_t st);
// launch_adapt for up to BMAX members, one launch per adaptation kernel;
// S2 is a second sort scratch (at least B keys) so two sorts share launches
struct AdaptMember {
  Dev D;
  SortScratch S, S2;
  uint32_t *keys, *vals, *keys2, *vals2;
};
void launch_adapt_batch(const AdaptMember *m, int n, int sms, cudaStream_t st);
void launch_stats(const Dev &D, cudaStream_t st);
void launch_fields_to_dense(const Dev &D, const void *src, int mode, float *dst, cudaStream_t st);
void launch_h16_to_f32(const uint16_t *src, float *dst, long long n, int mode, cudaStream_t st);
void launch_f32_to_h16(const float *src, uint16_t *dst, long long n, int mode, cudaStream_t st);
void launch_apron_table(const Dev &D, long long *dst, cudaStream_t st);

// k_adjoint.cu — transpose of one step's density map (flow and topology fixed)
void launch_adjoint_step(const Dev &D, float *lam_in_scratch, float *lam_out, float *lam_em, int sms,
                         cudaStream_t st);
void launch_adjoint_dense(const Dev &D, const float *lam_dense, float *lam, cudaStream_t st);
// Full adjoint of one step (planes of nc = 64 * max_blocks cells). Phase A
// runs on the state after the step (DA: its topology, projected velocity,
// and as scalars those its advection read), phase B on the state before it
// (D0: topology, velocity, scalars and fluidity of its start).
struct AdjFull {
  float *lv;               // 3 planes: adjoint of the velocity, after the step in, worked in place
  float *lq;               // nq planes: adjoint of the scalars after the step, worked in place
  float *lp0, *lp1, *ld;   // adjoint of p, p~ and div in the transposed cascade (consecutive planes)
  float *out_v, *out_q;    // 3 and nq planes: adjoint of the state before the step
};
void launch_adjoint_full_phase_a(const Dev &DA, const AdjFull &A, float *lam_em, int sweeps, int sms,
                                 cudaStream_t st);
void launch_adjoint_full_phase_b(const Dev &D0, const AdjFull &A, cudaStream_t st);

// k_render.cu — headless ray marcher (parameters mirror dcg_render_params)
struct RenderP {
  int width, height, aa, channel, shadows, solids, precise, pad;
  float eye[3], eye_dir[3], fov, sun[3], ambient, smoke[3], scene[3], floor_[3];
};

// k_uniform.cu — uniform (dense, mip-mapped) grid
struct UDev {
  int gx, gy, gz, levels, nq, ref_compat, pad0, pad1;
  long long nc, nmip;
  long long mip_off[MAXL];
  Phys ph;
  Geom g;  // gx/gy/gz for the shared boundary-condition helpers
  float *q[3], *tq[3], *v[3], *tv[3];
  float *w, *p, *pt, *div;
  double *red;
};
void launch_u_fluidity(const UDev &U, cudaStream_t st);
void launch_u_sources(const UDev &U, cudaStream_t st);
void launch_u_advect_velocity(const UDev &U, cudaStream_t st);
void launch_u_advect_scalars(const UDev &U, cudaStream_t st);
void launch_u_project(const UDev &U, int top_pairs, int pairs, bool local, cudaStream_t st);
void launch_u_add_noise(const UDev &U, unsigned long long seed, float amp, cudaStream_t st);
void launch_u_stats(const UDev &U, cudaStream_t st);
void launch_render_adaptive(const Dev &D, const RenderP &R, float4 *out, cudaStream_t st);
void launch_render_uniform(const UDev &U, const RenderP &R, float4 *out, cudaStream_t st);

}  // namespace dcg
