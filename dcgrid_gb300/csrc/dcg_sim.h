// dcg_sim.h — the simulation handle behind the C ABI (internal).
//
// Mirrors the reference's FluidSimulationDCGrid / FluidSimulationUniform
// objects (src/dcgrid/fluid_simulation_dcgrid.cu, src/uniformgrid/
// fluid_simulation_uniform.cu): the handle owns its device memory, the budget
// split and level derivation follow the reference, and the step is the
// reference's stage order.
#pragma once
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/dcg.h"
#include "dcg_kernels.h"

using namespace dcg;

namespace {

int idiv_up(int a, int b) { return (a % b != 0) ? (a / b + 1) : (a / b); }

}  // namespace

struct dcg_sim {
  dcg_params P{};
  int mode = DCG_MODE_ADAPTIVE;
  std::string err;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int device = 0, sms = 148;
  std::vector<void *> allocs;
  size_t bytes = 0;
  bool failed = false;
  long long steps = 0;

  // adaptive
  Dev D{};
  SortScratch S{};
  uint32_t *keys = nullptr, *vals = nullptr, *keys2 = nullptr, *vals2 = nullptr;
  float *dense_tmp = nullptr;
  float *emis = nullptr;  // emission_n^3 field
  long long *apron_tmp = nullptr;
  float *vbuf[2][3] = {}, *qbuf[2][3] = {};
  uint16_t *qhbuf[2][3] = {};  // 16-bit scalar storage (mixed precision)
  float *conv_tmp = nullptr;   // FP32 staging for access to 16-bit fields
  float *adj_tmp = nullptr;    // adjoint scratch (allocated on first use)
  // full adjoint scratch (first use): 19 planes (the state before the step,
  // the scalars the advection read, the adjoint planes) and a copy of the
  // block table of the step's start
  float *afull = nullptr;
  int4 *afull_pos = nullptr;
  uint32_t *afull_parent = nullptr, *afull_child = nullptr, *afull_nbr = nullptr;
  float *render_tmp = nullptr; // renderer output staging for host buffers
  size_t render_cap = 0;
  float *hmap = nullptr;       // terrain heightmap (dcg_set_heightmap), or null
  int hm_nx = 0, hm_nz = 0;
  int vpar = 0, qpar = 0;

  // uniform
  UDev U{};
  float *uvbuf[2][3] = {}, *uqbuf[2][3] = {};

  // graphs keyed by (vpar, qpar)
  std::map<int, cudaGraphExec_t> graphs;
  bool use_graphs = true;
  long long kernels_per_step = 0;
  int ls_grid = 0;  // CTAs of the cooperative level solve (0 = per-sweep launches)
  // level solve kernel: 3 = the staged solve shared with batches (two-level
  // barrier); 2 = the per-level kernel with a two-level barrier, taken when
  // the staged solve's cooperative grid cannot be formed on the device
  int ls_epoch = 3;
  int ls_grid_staged = 0;  // CTAs of the staged solve
  // level solve of single simulations: pipelined staged sweeps, two tile buffers,
  // block descriptions cached in 3 x 8 KB of shared memory when they fit.
  // Variant 19 (3 CTAs per SM, two blocks per claim); variant 83 (4 CTAs per
  // SM, one block per claim) measured faster on the 256^3 cloud (1.85 against
  // 1.93 ms per step) but slower on the 16 plumes stepped as single
  // simulations (27.3 against 26.5 ms) and on the reference-default scenes
  // (2.01 / 4.00 against 1.99 / 3.89 ms per step).
  static constexpr int kSolveVariant = 19;
  // batch members: p and p~ are slices of the batch's arenas, and the batch
  // steps the member (its own step and stage entry points are refused)
  float *ext_p = nullptr, *ext_pt = nullptr, *ext_div = nullptr;
  float *ext_emis = nullptr;  // batch members: the emission map is a slice of the batch's arena
  // batch members with defect correction: residual, correction and its
  // ping-pong plane are slices of the batch's arenas, the norms of its array
  float *ext_rr = nullptr, *ext_e = nullptr, *ext_et = nullptr;
  double *ext_dnorm = nullptr;
  bool batch_member = false;

  int fail(int code, const std::string &msg) {
    err = msg;
    return code;
  }
  int cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return DCG_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    failed = true;
    return DCG_E_CUDA;
  }
  // plan_only: creation only adds up the device bytes it would allocate
  // (no CUDA calls), for the memory-budget calculator
  bool plan_only = false;
  template <typename T> int alloc(T **p, size_t count) {
    void *q = nullptr;
    const size_t nbytes = std::max<size_t>(count * sizeof(T), 256);
    if (plan_only) {
      bytes += nbytes;
      *p = nullptr;
      return DCG_OK;
    }
    cudaError_t e = cudaMalloc(&q, nbytes);
    if (e != cudaSuccess) return cuda(e, "cudaMalloc");
    allocs.push_back(q);
    bytes += nbytes;
    *p = reinterpret_cast<T *>(q);
    return DCG_OK;
  }
  void free_all() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
    bytes = 0;
  }
  ~dcg_sim() {
    if (render_tmp) cudaFree(render_tmp);
    if (hmap) cudaFree(hmap);
    free_all();
    if (own_stream && stream) cudaStreamDestroy(stream);
  }

  void bind_parity() {
    for (int d = 0; d < 3; d++) {
      D.v[d] = vbuf[vpar][d];
      D.tv[d] = vbuf[vpar ^ 1][d];
      U.v[d] = uvbuf[vpar][d];
      U.tv[d] = uvbuf[vpar ^ 1][d];
    }
    for (int k = 0; k < 3; k++) {
      D.q[k] = qbuf[qpar][k];
      D.tq[k] = qbuf[qpar ^ 1][k];
      D.qh[k] = qhbuf[qpar][k];
      D.tqh[k] = qhbuf[qpar ^ 1][k];
      U.q[k] = uqbuf[qpar][k];
      U.tq[k] = uqbuf[qpar ^ 1][k];
    }
  }

  void fill_phys(Phys &ph) {
    ph.dt = P.dt;
    ph.dx = P.dx;
    ph.rdx = 1.f / P.dx;
    ph.inlet = P.inlet_enabled;
    ph.v_emit = P.velocity_emission_rate;
    ph.d_emit = P.density_emission_rate;
    ph.emit_radius = P.emission_radius;
    ph.solids = P.solids;
    ph.sphere_r = P.sphere_radius_world;
    ph.criterion = P.refine_criterion;
    ph.refine_threshold = P.refine_threshold;
    ph.vort_t = P.vort_threshold;
    ph.grad_t = P.grad_threshold;
    ph.buoy_a = P.buoy_alpha;
    ph.buoy_b = P.buoy_beta;
    ph.t_amb = P.t_ambient;
    ph.src = P.src_enabled;
    for (int i = 0; i < 3; i++) {
      ph.src_c[i] = P.src_center[i];
      ph.wind_v[i] = P.wind[i];
    }
    ph.src_r = P.src_radius;
    ph.src_val[0] = P.src_density;
    ph.src_val[1] = P.src_temperature;
    ph.src_val[2] = P.src_vapor;
    ph.src_jit = P.src_jitter;
    ph.src_seed = P.src_jitter_seed;
    ph.wind = P.wind_enabled;
    ph.ter_amp = P.terrain_amplitude;
    ph.ter_base = P.terrain_base_height;
    ph.ter_freq = P.terrain_frequency;
    ph.ter_pers = P.terrain_persistence;
    ph.ter_oct = P.terrain_octaves;
    ph.ter_seed = P.terrain_seed;
    ph.em_n = P.emission_n;
    ph.em_band = P.emission_band;
    ph.em = emis;
    ph.hm = hmap;
    ph.hm_nx = hm_nx;
    ph.hm_nz = hm_nz;
    ph.hm_sx = hmap ? (float)hm_nx / (float)P.gx : 0.f;
    ph.hm_sz = hmap ? (float)hm_nz / (float)P.gz : 0.f;
  }

  int validate_common() {
    if (P.gx <= 0 || P.gy <= 0 || P.gz <= 0) return fail(DCG_E_INVALID, "domain must be positive");
    if (!(P.dx > 0.f)) return fail(DCG_E_INVALID, "dx must be positive");
    if (P.jacobi_iters < 0 || (P.jacobi_iters & 1))
      return fail(DCG_E_INVALID, "jacobi_iters must be even and >= 0");
    if (P.n_scalars != 1 && P.n_scalars != 3) return fail(DCG_E_INVALID, "n_scalars must be 1 or 3");
    if (P.precision != DCG_PRECISION_FP32 && P.precision != DCG_PRECISION_MIXED &&
        P.precision != DCG_PRECISION_MIXED_FP16)
      return fail(DCG_E_INVALID, "unknown precision");
    if (P.defect_passes < 0 || P.defect_passes > 16) return fail(DCG_E_INVALID, "defect_passes must be in [0, 16]");
    return DCG_OK;
  }

  // ---------------------------------------------------------------- adaptive
  // Level derivation and budget split: fluid_simulation_dcgrid.cu:12-69.
  int create_adaptive() {
    int rc = validate_common();
    if (rc) return rc;
    Geom &g = D.g;
    std::memset(&g, 0, sizeof(g));
    g.gx = P.gx; g.gy = P.gy; g.gz = P.gz;
    const int minDim = std::min(P.gx, std::min(P.gy, P.gz));
    int cellSize = 2, levels = 1;
    while (P.gx % cellSize == 0 && P.gy % cellSize == 0 && P.gz % cellSize == 0 && cellSize * BW <= minDim) {
      levels++;
      cellSize *= 2;
    }
    if (P.levels > 0) levels = P.levels;
    if (levels > MAXL) return fail(DCG_E_INVALID, "at most 16 levels");
    const int ext = BW << (levels - 1);
    if (P.gx % ext || P.gy % ext || P.gz % ext)
      return fail(DCG_E_INVALID, "domain must be a multiple of the coarsest block extent");
    g.levels = levels;
    for (int l = 0, cs = 1; l < levels; l++, cs *= 2) {
      g.rx[l] = idiv_up(P.gx, cs * BW);
      g.ry[l] = idiv_up(P.gy, cs * BW);
      g.rz[l] = idiv_up(P.gz, cs * BW);
      g.full[l] = (long long)g.rx[l] * g.ry[l] * g.rz[l];
    }
    const long long B = P.max_blocks;
    if (B < g.full[levels - 1]) return fail(DCG_E_BUDGET, "too few blocks to fill the coarsest level");
    if (B >= (1ll << 28)) return fail(DCG_E_INVALID, "max_blocks must be below 2^28");
    g.budget[levels - 1] = g.full[levels - 1];
    long long left = B - g.budget[levels - 1];
    for (int l = levels - 2; l >= 0; l--) {
      g.budget[l] = std::min(left / (l + 1), g.full[l]);
      left -= g.budget[l];
    }
    if (g.budget[0] == 0) return fail(DCG_E_BUDGET, "too few blocks to reach the finest level");
    g.off[0] = 0;
    for (int l = 1; l < levels; l++) g.off[l] = g.off[l - 1] + g.budget[l - 1];
    g.sparse = 0;
    for (int l = 0; l < levels; l++)
      if (g.budget[l] < g.full[l]) g.sparse = l + 1;
    g.B = B;
    g.nq = P.n_scalars;
    g.ref_compat = P.ref_compat;
    g.mixed = P.precision == DCG_PRECISION_MIXED ? 1 : (P.precision == DCG_PRECISION_MIXED_FP16 ? 2 : 0);
    g.dpass = P.defect_passes;
    fill_phys(D.ph);

    const size_t nc = (size_t)B * BV;
    if ((rc = alloc(&D.pos, B))) return rc;
    if ((rc = alloc(&D.parent, B))) return rc;
    if ((rc = alloc(&D.child, 8 * B))) return rc;
    if ((rc = alloc(&D.nbr, 27 * B))) return rc;
    if ((rc = alloc(&D.flags, B))) return rc;
    if ((rc = alloc(&D.load, MAXL))) return rc;
    if ((rc = alloc(&D.move_limit, MAXL))) return rc;
    for (int par = 0; par < 2; par++) {
      for (int d = 0; d < 3; d++)
        if ((rc = alloc(&vbuf[par][d], nc))) return rc;
      for (int k = 0; k < P.n_scalars; k++) {
        if (g.mixed) {
          if ((rc = alloc(&qhbuf[par][k], nc))) return rc;
        } else if ((rc = alloc(&qbuf[par][k], nc))) {
          return rc;
        }
      }
    }
    if ((rc = alloc(&D.w, nc))) return rc;
    if (ext_p) {
      D.p = ext_p;
      D.pt = ext_pt;
    } else {
      if ((rc = alloc(&D.p, nc))) return rc;
      if ((rc = alloc(&D.pt, nc))) return rc;
    }
    if (ext_div) D.div = ext_div;
    else if ((rc = alloc(&D.div, nc))) return rc;
    if ((rc = alloc(&D.ss, 8 * B + 1))) return rc;
    if ((rc = alloc(&D.bs, B))) return rc;
    if ((rc = alloc(&D.moves, 2 * 2 * B))) return rc;
    if ((rc = alloc(&D.mold, 2 * B))) return rc;
    if ((rc = alloc(&D.refines, 2 * 2 * B))) return rc;
    if ((rc = alloc(&D.touched, 2 * B))) return rc;
    if ((rc = alloc(&D.ctr, C_COUNT))) return rc;
    if ((rc = alloc(&D.err, 4))) return rc;
    if ((rc = alloc(&D.red, 32))) return rc;
    if ((rc = alloc(&D.bar, 64 + 32 * 18))) return rc;
    if ((rc = alloc(&D.epoch, B))) return rc;
    if ((rc = alloc(&D.binfo, (long long)BI_WORDS * B))) return rc;
    if (P.defect_passes > 0) {
      if (ext_rr) {
        D.rr = ext_rr;
        D.e = ext_e;
        D.et = ext_et;
        D.dnorm = ext_dnorm;
      } else {
        if ((rc = alloc(&D.rr, nc))) return rc;
        if ((rc = alloc(&D.e, nc))) return rc;
        if ((rc = alloc(&D.et, nc))) return rc;
        if ((rc = alloc(&D.dnorm, 2 * (P.defect_passes + 1)))) return rc;
      }
    }
    if (plan_only) return plan_tail_adaptive(B);
    ls_grid = level_solve_grid(sms);
    ls_grid_staged = batch_solve_grid(sms, kSolveVariant, 0);
    if (ls_grid_staged <= 0 && ls_epoch == 3) ls_epoch = 2;
    if (P.emission_n > 0) {
      const size_t ne = (size_t)P.emission_n * P.emission_n * P.emission_n;
      if (ext_emis) emis = ext_emis;
      else if ((rc = alloc(&emis, ne))) return rc;
      if ((rc = cuda(cudaMemset(emis, 0, ne * 4), "emission"))) return rc;
      fill_phys(D.ph);
      fill_phys(U.ph);
    }
    const long long nsort = 8 * B;
    if ((rc = alloc(&keys, nsort))) return rc;
    if ((rc = alloc(&vals, nsort))) return rc;
    if ((rc = alloc(&keys2, nsort))) return rc;
    if ((rc = alloc(&vals2, nsort))) return rc;
    if ((rc = alloc(&S.k1, nsort))) return rc;
    if ((rc = alloc(&S.v1, nsort))) return rc;
    const long long nt = sort_tiles(nsort);
    if ((rc = alloc(&S.hist, 256 * nt))) return rc;
    if ((rc = alloc(&S.totals, 256))) return rc;
    if ((rc = alloc(&S.tile_sums, nt + 1))) return rc;
    S.max_n = nsort;
    bind_parity();
    return reset_adaptive();
  }

  // the allocations create_adaptive makes after the block table and fields
  int plan_tail_adaptive(long long B) {
    void *v;
    if (P.emission_n > 0) alloc(reinterpret_cast<float **>(&v), (size_t)P.emission_n * P.emission_n * P.emission_n);
    const long long nsort = 8 * B, nt = sort_tiles(nsort);
    for (int i = 0; i < 6; i++) alloc(reinterpret_cast<uint32_t **>(&v), nsort);
    alloc(reinterpret_cast<uint32_t **>(&v), 256 * nt);
    alloc(reinterpret_cast<uint32_t **>(&v), 256);
    alloc(reinterpret_cast<uint32_t **>(&v), nt + 1);
    return DCG_OK;
  }

  // FluidSimulationDCGrid::reset + init (fluid_simulation_dcgrid.cu:190-261)
  int reset_adaptive() {
    int rc;
    vpar = qpar = 0;
    bind_parity();
    const size_t nc = (size_t)D.g.B * BV;
    for (int par = 0; par < 2; par++) {
      for (int d = 0; d < 3; d++) cudaMemsetAsync(vbuf[par][d], 0, nc * 4, stream);
      for (int k = 0; k < P.n_scalars; k++) {
        if (qbuf[par][k]) cudaMemsetAsync(qbuf[par][k], 0, nc * 4, stream);
        if (qhbuf[par][k]) cudaMemsetAsync(qhbuf[par][k], 0, nc * 2, stream);
      }
    }
    cudaMemsetAsync(D.w, 0, nc * 4, stream);
    cudaMemsetAsync(D.p, 0, nc * 4, stream);
    cudaMemsetAsync(D.pt, 0, nc * 4, stream);
    cudaMemsetAsync(D.div, 0, nc * 4, stream);
    cudaMemsetAsync(D.nbr, 0xff, (size_t)27 * D.g.B * 4, stream);
    cudaMemsetAsync(D.ctr, 0, sizeof(long long) * C_COUNT, stream);
    cudaMemsetAsync(D.err, 0, 4, stream);
    cudaMemsetAsync(D.bar, 0, 4 * (64 + 32 * 18), stream);
    long long load[MAXL] = {0}, ml[MAXL] = {0};
    for (int l = 0; l < D.g.levels; l++) load[l] = D.g.budget[l] == D.g.full[l] ? D.g.budget[l] : 0;
    if ((rc = cuda(cudaMemcpyAsync(D.load, load, sizeof(load), cudaMemcpyHostToDevice, stream), "load"))) return rc;
    if ((rc = cuda(cudaMemcpyAsync(D.move_limit, ml, sizeof(ml), cudaMemcpyHostToDevice, stream), "ml"))) return rc;
    launch_init_blocks(D, stream);
    for (int l = D.g.sparse; l < D.g.levels; l++) launch_activate_level(D, l, stream);
    launch_build_nbr(D, false, stream);
    for (int i = 0; i < P.init_adapt_passes; i++) launch_adapt(D, S, keys, vals, keys2, vals2, sms, stream);
    if (P.src_enabled) {
      launch_sources(D, stream);
      restrict_q();
    }
    steps = 0;
    return sync("reset");
  }

  void restrict_v() {
    FieldList fl{};
    fl.n = 3;
    for (int d = 0; d < 3; d++) fl.f[d] = D.v[d];
    launch_restrict(D, fl, stream);
  }
  void restrict_q() {
    FieldList fl{};
    fl.n = P.n_scalars;
    for (int k = 0; k < P.n_scalars; k++) {
      fl.f[k] = D.g.mixed ? static_cast<void *>(D.qh[k]) : static_cast<void *>(D.q[k]);
      fl.mode[k] = D.g.mixed;
    }
    launch_restrict(D, fl, stream);
  }
  void restrict_div() {
    FieldList fl{};
    fl.n = 1;
    fl.f[0] = D.div;
    launch_restrict(D, fl, stream);
  }

  // stages (fluid_simulation_dcgrid.cu:263-346)
  // the cell stages through the batched launchers as a batch of one, staged
  // (one warp, or for the advections two warps, per block through shared tiles)
  void cells(int stage, int tile) {
    CellBatch C{};
    C.n = 1;
    C.d[0] = D;
    launch_cells_batch(stage, C, tile, stream, true);
  }
  void a_advect_velocity() {
    cells(0, 1);
    vpar ^= 1;
    bind_parity();
    restrict_v();
  }
  void a_adapt() { launch_adapt(D, S, keys, vals, keys2, vals2, sms, stream); }
  // apply = false leaves out the pressure application (and its restriction):
  // the step then runs it fused with the scalar advection (a_apply_advect)
  void a_project(bool local, bool apply = true) {
    cells(2, 1);
    restrict_div();
    const int top = D.g.levels - 1;
    if (ls_grid > 0) {
      // one cooperative launch per level: prolongation (not for the coarsest
      // level, nor in projectLocal) and all of the level's sweeps
      const int sweeps = local ? 2 * P.jacobi_iters : P.jacobi_iters;
      if (ls_epoch == 3) {
        for (int l = top; l >= 0; l--) solve_staged(l, local ? 0 : 1, sweeps);
        if (!local && P.defect_passes > 0) defect_correct(sweeps);
      } else {
        for (int l = top; l >= 0; l--)
          launch_level_solve(D, l, (!local && l < top) ? 1 : 0, sweeps, ls_grid, ls_epoch, stream);
      }
    } else if (local) {
      const int pairs = P.jacobi_iters;
      for (int l = top; l >= 0; l--)
        for (int i = 0; i < pairs; i++) {
          launch_jacobi(D, l, D.p, D.pt, stream);
          launch_jacobi(D, l, D.pt, D.p, stream);
        }
    } else {
      const int pairs = P.jacobi_iters / 2;
      for (int i = 0; i < pairs; i++) {
        launch_jacobi(D, top, D.p, D.pt, stream);
        launch_jacobi(D, top, D.pt, D.p, stream);
      }
      for (int l = top - 1; l >= 0; l--) {
        launch_prolongate(D, l, stream);
        for (int i = 0; i < pairs; i++) {
          launch_jacobi(D, l, D.p, D.pt, stream);
          launch_jacobi(D, l, D.pt, D.p, stream);
        }
      }
    }
    if (!apply) return;
    cells(3, 1);
    restrict_v();
  }
  // ---------------------------------------------------------------- state I/O
  // The state a step depends on, as (device pointer, bytes) sections in a
  // fixed order: block table, neighbour table, counters, then the fields of
  // the current buffer parity.
  std::vector<std::pair<void *, size_t>> state_sections() {
    std::vector<std::pair<void *, size_t>> s;
    const size_t B = (size_t)D.g.B, nc = B * BV;
    s.push_back({D.pos, B * sizeof(int4)});
    s.push_back({D.parent, B * 4});
    s.push_back({D.child, 8 * B * 4});
    s.push_back({D.nbr, 27 * B * 4});
    s.push_back({D.flags, B});
    s.push_back({D.load, MAXL * 8});
    s.push_back({D.move_limit, MAXL * 8});
    for (int d = 0; d < 3; d++) s.push_back({D.v[d], nc * 4});
    s.push_back({D.w, nc * 4});
    s.push_back({D.p, nc * 4});
    s.push_back({D.pt, nc * 4});
    s.push_back({D.div, nc * 4});
    for (int k = 0; k < P.n_scalars; k++)
      s.push_back({D.g.mixed ? static_cast<void *>(D.qh[k]) : static_cast<void *>(D.q[k]), nc * (D.g.mixed ? 2 : 4)});
    return s;
  }

  // FP64 defect correction after the cascade: per pass the FP64 residual of
  // every level's equations (norms into dnorm), the cascade on the residual
  // into e, and p += e; a last residual measures the result
  void defect_correct(int sweeps) {
    const int K = P.defect_passes, top = D.g.levels - 1;
    cudaMemsetAsync(D.dnorm, 0, sizeof(double) * 2 * (K + 1), stream);
    for (int k = 0; k <= K; k++) {
      CellBatch C{};  // the staged FP64 residual of pass k
      C.n = 1;
      C.arg = k;
      C.d[0] = D;
      launch_cells_batch(6, C, 1, stream);
      if (k == K) break;
      cudaMemsetAsync(D.e, 0, (size_t)D.g.B * BV * sizeof(float), stream);
      for (int l = top; l >= 0; l--) solve_staged(l, 1, sweeps, D.e, D.et, D.rr);
      launch_add_correction(D, stream);
    }
  }

  // one level of the cascade through the staged solve, as a batch of one
  // (prolongation only below the coarsest level), on p / p~ / div or on the
  // given planes
  void solve_staged(int level, int prolong, int sweeps, float *pp = nullptr, float *ppt = nullptr,
                    float *pdiv = nullptr) {
    SolveBatch SB{};
    SB.n = 1;
    SB.maxtop = D.g.levels - 1;
    SB.prolong = prolong;
    SB.p = pp ? pp : D.p;
    SB.pt = ppt ? ppt : D.pt;
    SB.div = pdiv ? pdiv : D.div;
    SB.binfo = D.binfo;
    SB.bar = D.bar;
    SB.err = D.err;
    SB.arena[0] = 0;
    SB.d[0] = D;
    if (pp) {  // the prolongation and the cached alpha*div read these through D
      SB.d[0].p = pp;
      SB.d[0].pt = ppt;
      SB.d[0].div = pdiv;
    }
    launch_level_solve_batch(SB, SB.maxtop - level, sweeps, ls_grid_staged, kSolveVariant, 1, stream);
  }
  void a_advect_scalars() {
    cells(1, 1);
    qpar ^= 1;
    bind_parity();
    restrict_q();
  }
  // pressure application and scalar advection in one staged pass (cell
  // stage 5), then the restriction of velocity and scalars in one pass: the
  // results of cells(3) + restrict_v() + a_advect_scalars()
  void a_apply_advect() {
    cells(5, 1);
    qpar ^= 1;
    bind_parity();
    FieldList fl{};
    fl.n = 3 + P.n_scalars;
    for (int d = 0; d < 3; d++) fl.f[d] = D.v[d];
    for (int k = 0; k < P.n_scalars; k++) {
      fl.f[3 + k] = D.g.mixed ? static_cast<void *>(D.qh[k]) : static_cast<void *>(D.q[k]);
      fl.mode[3 + k] = D.g.mixed;
    }
    launch_restrict(D, fl, stream);
  }

  // ---------------------------------------------------------------- uniform
  int create_uniform() {
    int rc = validate_common();
    if (rc) return rc;
    if (P.defect_passes) return fail(DCG_E_INVALID, "defect correction is implemented for the adaptive grid");
    std::memset(&U, 0, sizeof(U));
    U.gx = P.gx; U.gy = P.gy; U.gz = P.gz;
    const int minDim = std::min(P.gx, std::min(P.gy, P.gz));
    int cellSize = 2, levels = 1;
    while (P.gx % cellSize == 0 && P.gy % cellSize == 0 && P.gz % cellSize == 0 && cellSize * 4 <= minDim) {
      levels++;
      cellSize *= 2;
    }
    if (P.levels > 0) levels = P.levels;
    if (levels > MAXL) return fail(DCG_E_INVALID, "at most 16 levels");
    const int top = 1 << (levels - 1);
    if (P.gx % top || P.gy % top || P.gz % top)
      return fail(DCG_E_INVALID, "domain must be divisible by 2^(levels-1)");
    U.levels = levels;
    U.nq = P.n_scalars;
    U.ref_compat = P.ref_compat;
    U.nc = (long long)P.gx * P.gy * P.gz;
    long long o = 0;
    for (int l = 0; l < levels; l++) {
      U.mip_off[l] = o;
      const long long s = 1ll << l;
      o += U.nc / (s * s * s);
    }
    U.nmip = o;
    fill_phys(U.ph);
    std::memset(&U.g, 0, sizeof(U.g));
    U.g.gx = P.gx; U.g.gy = P.gy; U.g.gz = P.gz;
    for (int par = 0; par < 2; par++) {
      for (int d = 0; d < 3; d++)
        if ((rc = alloc(&uvbuf[par][d], U.nc))) return rc;
      for (int k = 0; k < P.n_scalars; k++)
        if ((rc = alloc(&uqbuf[par][k], U.nc))) return rc;
    }
    if ((rc = alloc(&U.w, U.nmip))) return rc;
    if ((rc = alloc(&U.p, U.nmip))) return rc;
    if ((rc = alloc(&U.pt, U.nmip))) return rc;
    if ((rc = alloc(&U.div, U.nmip))) return rc;
    if ((rc = alloc(&U.red, 32))) return rc;
    if (P.emission_n > 0) {
      const size_t ne = (size_t)P.emission_n * P.emission_n * P.emission_n;
      if ((rc = alloc(&emis, ne))) return rc;
      if (plan_only) return DCG_OK;
      if ((rc = cuda(cudaMemset(emis, 0, ne * 4), "emission"))) return rc;
      fill_phys(D.ph);
      fill_phys(U.ph);
    }
    if (plan_only) return DCG_OK;
    bind_parity();
    return reset_uniform();
  }
  // FluidSimulationUniform::reset / init (fluid_simulation_uniform.cu:76-92)
  int reset_uniform() {
    vpar = qpar = 0;
    bind_parity();
    for (int par = 0; par < 2; par++) {
      for (int d = 0; d < 3; d++) cudaMemsetAsync(uvbuf[par][d], 0, U.nc * 4, stream);
      for (int k = 0; k < P.n_scalars; k++) cudaMemsetAsync(uqbuf[par][k], 0, U.nc * 4, stream);
    }
    cudaMemsetAsync(U.w, 0, U.nmip * 4, stream);
    cudaMemsetAsync(U.p, 0, U.nmip * 4, stream);
    cudaMemsetAsync(U.pt, 0, U.nmip * 4, stream);
    cudaMemsetAsync(U.div, 0, U.nmip * 4, stream);
    launch_u_fluidity(U, stream);
    if (P.src_enabled) launch_u_sources(U, stream);
    steps = 0;
    return sync("reset");
  }
  void u_advect_velocity() {
    launch_u_advect_velocity(U, stream);
    vpar ^= 1;
    bind_parity();
  }
  void u_project(bool local) {
    const int top_pairs = P.ref_compat ? 2 : P.jacobi_iters / 2;
    const int pairs = local ? (P.ref_compat ? 5 : P.jacobi_iters / 2) : (P.ref_compat ? 1 : P.jacobi_iters / 2);
    launch_u_project(U, top_pairs, pairs, local, stream);
  }
  void u_advect_scalars() {
    launch_u_advect_scalars(U, stream);
    qpar ^= 1;
    bind_parity();
  }

  // ---------------------------------------------------------------- common
  int sync(const char *what) {
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    return cuda(e, what);
  }
  int check_launch(const char *what) { return cuda(cudaGetLastError(), what); }

  void stage_advect_velocity() { mode == DCG_MODE_ADAPTIVE ? a_advect_velocity() : u_advect_velocity(); }
  void stage_adapt() {
    if (mode == DCG_MODE_ADAPTIVE) a_adapt();
    else launch_u_fluidity(U, stream);  // FluidSimulationUniform::adaptTopology
  }
  void stage_project(bool local) { mode == DCG_MODE_ADAPTIVE ? a_project(local) : u_project(local); }
  void stage_advect_scalars() { mode == DCG_MODE_ADAPTIVE ? a_advect_scalars() : u_advect_scalars(); }
  void step_once() {
    stage_advect_velocity();
    stage_adapt();
    if (mode == DCG_MODE_ADAPTIVE) {
      a_project(false, false);
      a_apply_advect();
    } else {
      stage_project(false);
      stage_advect_scalars();
    }
  }

  int step(int n) {
    for (int i = 0; i < n; i++) {
      if (use_graphs) {
        const int key = vpar * 2 + qpar;
        auto it = graphs.find(key);
        if (it == graphs.end()) {
          cudaGraph_t g = nullptr;
          int rc;
          if ((rc = cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capture"))) return rc;
          step_once();
          if ((rc = cuda(cudaStreamEndCapture(stream, &g), "end capture"))) return rc;
          size_t nn = 0;
          if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn > 0) {
            std::vector<cudaGraphNode_t> nodes(nn);
            cudaGraphGetNodes(g, nodes.data(), &nn);
            long long nk = 0;
            for (auto nd : nodes) {
              cudaGraphNodeType t;
              if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) nk++;
            }
            kernels_per_step = nk;
          }
          cudaGraphExec_t ge = nullptr;
          if ((rc = cuda(cudaGraphInstantiate(&ge, g, 0), "instantiate"))) {
            cudaGraphDestroy(g);
            return rc;
          }
          cudaGraphDestroy(g);
          graphs[key] = ge;
          // step_once() advanced the buffer parities while capturing
          if ((rc = cuda(cudaGraphLaunch(ge, stream), "graph launch"))) return rc;
        } else {
          int rc;
          if ((rc = cuda(cudaGraphLaunch(it->second, stream), "graph launch"))) return rc;
          vpar ^= 1;
          qpar ^= 1;
          bind_parity();
        }
      } else {
        step_once();
        int rc;
        if ((rc = check_launch("step"))) return rc;
      }
      steps++;
    }
    return check_launch("step");
  }
};
