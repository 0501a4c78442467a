// dcg_api.cu — host implementation of the C ABI in include/dcg.h.
//
// Mirrors the reference's FluidSimulationDCGrid / FluidSimulationUniform
// objects (src/dcgrid/fluid_simulation_dcgrid.cu, src/uniformgrid/
// fluid_simulation_uniform.cu): the handle owns its device memory, the budget
// split and level derivation follow the reference, and the step is the
// reference's stage order. Differences: no exit(), status codes instead;
// no host round trips inside a step; every launch goes to the handle's
// stream, and dcg_step replays a captured CUDA graph of the whole step.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
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
  int vpar = 0, qpar = 0;

  // uniform
  UDev U{};
  float *uvbuf[2][3] = {}, *uqbuf[2][3] = {};

  // graphs keyed by (vpar, qpar)
  std::map<int, cudaGraphExec_t> graphs;
  bool use_graphs = true;
  long long kernels_per_step = 0;
  int ls_grid = 0;  // CTAs of the cooperative level solve (0 = per-sweep launches)
  int ls_epoch = 2; // sweep ordering: 0 flat grid barrier, 1 neighbour epochs, 2 two-level barrier

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
  template <typename T> int alloc(T **p, size_t count) {
    void *q = nullptr;
    const size_t nbytes = std::max<size_t>(count * sizeof(T), 256);
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
    if ((rc = alloc(&D.p, nc))) return rc;
    if ((rc = alloc(&D.pt, nc))) return rc;
    if ((rc = alloc(&D.div, nc))) return rc;
    if ((rc = alloc(&D.ss, 8 * B + 1))) return rc;
    if ((rc = alloc(&D.bs, B))) return rc;
    if ((rc = alloc(&D.moves, 2 * 2 * B))) return rc;
    if ((rc = alloc(&D.refines, 2 * 2 * B))) return rc;
    if ((rc = alloc(&D.touched, 2 * B))) return rc;
    if ((rc = alloc(&D.ctr, C_COUNT))) return rc;
    if ((rc = alloc(&D.err, 4))) return rc;
    if ((rc = alloc(&D.red, 32))) return rc;
    if ((rc = alloc(&D.bar, 64 + 32 * 18))) return rc;
    if ((rc = alloc(&D.epoch, B))) return rc;
    ls_grid = level_solve_grid(sms);
    if (const char *m = std::getenv("DCG_SOLVE_SYNC"))
      ls_epoch = std::strcmp(m, "epoch") == 0 ? 1 : (std::strcmp(m, "barrier") == 0 ? 0 : 2);
    if (P.emission_n > 0) {
      const size_t ne = (size_t)P.emission_n * P.emission_n * P.emission_n;
      if ((rc = alloc(&emis, ne))) return rc;
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
  void a_advect_velocity() {
    launch_advect_velocity(D, stream);
    vpar ^= 1;
    bind_parity();
    restrict_v();
  }
  void a_adapt() { launch_adapt(D, S, keys, vals, keys2, vals2, sms, stream); }
  void a_project(bool local) {
    launch_divergence(D, stream);
    restrict_div();
    const int top = D.g.levels - 1;
    if (ls_grid > 0) {
      // one cooperative launch per level: prolongation (not for the coarsest
      // level, nor in projectLocal) and all of the level's sweeps
      const int sweeps = local ? 2 * P.jacobi_iters : P.jacobi_iters;
      for (int l = top; l >= 0; l--) launch_level_solve(D, l, (!local && l < top) ? 1 : 0, sweeps, ls_grid, ls_epoch, stream);
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
    launch_apply_pressure(D, stream);
    restrict_v();
  }
  void a_advect_scalars() {
    launch_advect_scalars(D, stream);
    qpar ^= 1;
    bind_parity();
    restrict_q();
  }

  // ---------------------------------------------------------------- uniform
  int create_uniform() {
    int rc = validate_common();
    if (rc) return rc;
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
      if ((rc = cuda(cudaMemset(emis, 0, ne * 4), "emission"))) return rc;
      fill_phys(D.ph);
      fill_phys(U.ph);
    }
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
    stage_project(false);
    stage_advect_scalars();
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

static int bad(dcg_sim *s) { return s == nullptr; }

extern "C" {

void dcg_default_params(dcg_params *p, int32_t gx, int32_t gy, int32_t gz, int64_t max_blocks) {
  std::memset(p, 0, sizeof(*p));
  p->gx = gx; p->gy = gy; p->gz = gz;
  p->levels = 0;
  p->max_blocks = max_blocks;
  p->dt = 3.f;  // src/data/sim_params.cpp:9-15
  p->dx = 10000.f / (float)gx;
  p->inlet_enabled = 1;
  p->velocity_emission_rate = 150.f;
  p->density_emission_rate = 0.002f;
  p->emission_radius = 750.f;
  p->solids = DCG_SOLIDS_NONE;
  p->sphere_radius_world = 2000.f;  // src/sdf.cuh:12
  p->jacobi_iters = 10;             // 5 pairs, fluid_simulation_dcgrid.cu:274-290
  p->init_adapt_passes = 5;         // fluid_simulation_dcgrid.cu:207-209
  p->refine_criterion = DCG_REFINE_GEOMETRIC;
  p->refine_threshold = 1e-4f;      // fluid_simulation_dcgrid.cu:461
  p->vort_threshold = 0.5f;
  p->grad_threshold = 0.05f;
  p->ref_compat = 1;
  p->n_scalars = 1;
  p->terrain_frequency = 1.f / 64.f;
  p->terrain_persistence = 0.5f;
  p->terrain_octaves = 5;
  p->precision = DCG_PRECISION_FP32;
}

int dcg_create(const dcg_params *params, int32_t mode, dcg_sim **out) {
  if (!params || !out) return DCG_E_INVALID;
  *out = nullptr;
  dcg_sim *s = new dcg_sim();
  s->P = *params;
  s->mode = mode;
  if (mode != DCG_MODE_ADAPTIVE && mode != DCG_MODE_UNIFORM) {
    delete s;
    return DCG_E_INVALID;
  }
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete s;
    return DCG_E_CUDA;
  }
  s->own_stream = true;
  if (params->precision != DCG_PRECISION_FP32 && mode == DCG_MODE_UNIFORM) {
    delete s;
    return DCG_E_INVALID;  // 16-bit scalar storage is implemented for the adaptive grid
  }
  const int rc = mode == DCG_MODE_ADAPTIVE ? s->create_adaptive() : s->create_uniform();
  if (rc) {
    delete s;
    return rc;
  }
  *out = s;
  return DCG_OK;
}

int dcg_destroy(dcg_sim *sim) {
  if (!sim) return DCG_E_INVALID;
  cudaStreamSynchronize(sim->stream);
  delete sim;
  return DCG_OK;
}

int dcg_reset(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  return s->mode == DCG_MODE_ADAPTIVE ? s->reset_adaptive() : s->reset_uniform();
}

int dcg_set_params(dcg_sim *s, const dcg_params *p) {
  if (bad(s) || !p) return DCG_E_INVALID;
  if (p->gx != s->P.gx || p->gy != s->P.gy || p->gz != s->P.gz || p->levels != s->P.levels ||
      p->max_blocks != s->P.max_blocks || p->n_scalars != s->P.n_scalars || p->precision != s->P.precision ||
      p->ref_compat != s->P.ref_compat)
    return s->fail(DCG_E_INVALID, "geometry, budget, scalars, precision and compat mode are fixed at creation");
  if (p->jacobi_iters < 0 || (p->jacobi_iters & 1)) return s->fail(DCG_E_INVALID, "jacobi_iters must be even");
  if (p->emission_n != s->P.emission_n) return s->fail(DCG_E_INVALID, "emission_n is fixed at creation");
  const Phys before = s->mode == DCG_MODE_ADAPTIVE ? s->D.ph : s->U.ph;
  const int iters_before = s->P.jacobi_iters;
  s->P = *p;
  s->fill_phys(s->D.ph);
  s->fill_phys(s->U.ph);
  const Phys &after = s->mode == DCG_MODE_ADAPTIVE ? s->D.ph : s->U.ph;
  // captured step graphs hold the physics by value: drop them only on change
  if (std::memcmp(&before, &after, sizeof(Phys)) != 0 || iters_before != p->jacobi_iters) {
    cudaStreamSynchronize(s->stream);
    for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
  }
  return DCG_OK;
}

int dcg_set_mode(dcg_sim **sim, int32_t mode) {
  if (!sim || !*sim) return DCG_E_INVALID;
  dcg_params p = (*sim)->P;
  dcg_sim *n = nullptr;
  const int rc = dcg_create(&p, mode, &n);
  if (rc) return rc;
  dcg_destroy(*sim);
  *sim = n;
  return DCG_OK;
}

int dcg_set_stream(dcg_sim *s, void *cuda_stream) {
  if (bad(s)) return DCG_E_INVALID;
  cudaStreamSynchronize(s->stream);
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->own_stream = false;
  s->stream = reinterpret_cast<cudaStream_t>(cuda_stream);
  return DCG_OK;
}

int dcg_get_info(const dcg_sim *s, dcg_info *info) {
  if (!s || !info) return DCG_E_INVALID;
  std::memset(info, 0, sizeof(*info));
  info->mode = s->mode;
  info->n_scalars = s->P.n_scalars;
  info->device_bytes = (int64_t)s->bytes;
  if (s->mode == DCG_MODE_ADAPTIVE) {
    info->levels = s->D.g.levels;
    info->sparse_levels = s->D.g.sparse;
    info->max_blocks = s->D.g.B;
    info->num_cells = s->D.g.B * BV;
    for (int l = 0; l < s->D.g.levels; l++) {
      info->full_blocks[l] = s->D.g.full[l];
      info->budget[l] = s->D.g.budget[l];
      info->offset[l] = s->D.g.off[l];
    }
  } else {
    info->levels = s->U.levels;
    info->num_cells = s->U.nc;
  }
  return DCG_OK;
}

const char *dcg_last_error_string(const dcg_sim *s) { return s ? s->err.c_str() : "null handle"; }

int dcg_step(dcg_sim *s, int32_t n) {
  if (bad(s) || n < 0) return DCG_E_INVALID;
  return s->step(n);
}
int dcg_advect_velocity(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  s->stage_advect_velocity();
  return s->check_launch("advect_velocity");
}
int dcg_adapt(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  s->stage_adapt();
  return s->check_launch("adapt");
}
int dcg_project(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  s->stage_project(false);
  return s->check_launch("project");
}
int dcg_project_local(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  s->stage_project(true);
  return s->check_launch("project_local");
}
int dcg_advect_scalars(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  s->stage_advect_scalars();
  return s->check_launch("advect_scalars");
}
int dcg_sync(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  int rc = s->sync("sync");
  if (rc) return rc;
  if (s->mode == DCG_MODE_ADAPTIVE) {
    uint32_t e = 0;
    if ((rc = s->cuda(cudaMemcpy(&e, s->D.err, 4, cudaMemcpyDeviceToHost), "err word"))) return rc;
    if (e) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "device error word 0x%x", e);
      return s->fail(DCG_E_DEVICE, buf);
    }
  }
  return DCG_OK;
}

int dcg_set_emission(dcg_sim *s, const float *field, int32_t where) {
  if (bad(s) || !field) return DCG_E_INVALID;
  if (!s->emis) return s->fail(DCG_E_INVALID, "created with emission_n = 0");
  const size_t n = (size_t)s->P.emission_n * s->P.emission_n * s->P.emission_n;
  return s->cuda(cudaMemcpyAsync(s->emis, field, n * 4,
                                 where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s->stream),
                 "set_emission");
}

int dcg_add_velocity_noise(dcg_sim *s, uint64_t seed, float amplitude) {
  if (bad(s)) return DCG_E_INVALID;
  if (s->mode == DCG_MODE_ADAPTIVE) launch_add_noise(s->D, seed, amplitude, s->stream);
  else launch_u_add_noise(s->U, seed, amplitude, s->stream);
  return s->check_launch("noise");
}

// A field's storage: pointer and format (0 FP32, 1 BF16, 2 FP16).
struct FieldRef {
  void *p;
  int mode;
};
static FieldRef field_ref(dcg_sim *s, int f) {
  const bool a = s->mode == DCG_MODE_ADAPTIVE;
  const int m = a ? s->D.g.mixed : 0;
  auto scalar = [&](int k) -> FieldRef {
    if (k >= s->P.n_scalars) return {nullptr, 0};
    if (!a) return {s->U.q[k], 0};
    return m ? FieldRef{s->D.qh[k], m} : FieldRef{s->D.q[k], 0};
  };
  switch (f) {
    case DCG_FIELD_DENSITY: return scalar(0);
    case DCG_FIELD_VEL_X: return {a ? s->D.v[0] : s->U.v[0], 0};
    case DCG_FIELD_VEL_Y: return {a ? s->D.v[1] : s->U.v[1], 0};
    case DCG_FIELD_VEL_Z: return {a ? s->D.v[2] : s->U.v[2], 0};
    case DCG_FIELD_FLUIDITY: return {a ? s->D.w : s->U.w, 0};
    case DCG_FIELD_PRESSURE: return {a ? s->D.p : s->U.p, 0};
    case DCG_FIELD_PRESSURE_TMP: return {a ? s->D.pt : s->U.pt, 0};
    case DCG_FIELD_DIVERGENCE: return {a ? s->D.div : s->U.div, 0};
    case DCG_FIELD_TEMPERATURE: return scalar(1);
    case DCG_FIELD_VAPOR: return scalar(2);
  }
  return {nullptr, 0};
}
static size_t field_cells(dcg_sim *s) {
  return s->mode == DCG_MODE_ADAPTIVE ? (size_t)s->D.g.B * BV : (size_t)s->U.nc;
}

int dcg_get_field(dcg_sim *s, int32_t field, float *dst, int32_t where) {
  if (bad(s) || !dst) return DCG_E_INVALID;
  const FieldRef r = field_ref(s, field);
  if (!r.p) return s->fail(DCG_E_NOT_FOUND, "no such field");
  const size_t cells = field_cells(s), n = cells * sizeof(float);
  int rc;
  const float *src = static_cast<const float *>(r.p);
  if (r.mode) {  // 16-bit storage: widen into an FP32 staging buffer
    if (!s->conv_tmp && (rc = s->alloc(&s->conv_tmp, cells))) return rc;
    launch_h16_to_f32(static_cast<const uint16_t *>(r.p), s->conv_tmp, (long long)cells, r.mode, s->stream);
    src = s->conv_tmp;
  }
  rc = s->cuda(cudaMemcpyAsync(dst, src, n, where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                               s->stream), "get_field");
  if (rc) return rc;
  return s->sync("get_field");
}
int dcg_set_field(dcg_sim *s, int32_t field, const float *src, int32_t where) {
  if (bad(s) || !src) return DCG_E_INVALID;
  const FieldRef r = field_ref(s, field);
  if (!r.p) return s->fail(DCG_E_NOT_FOUND, "no such field");
  const size_t cells = field_cells(s), n = cells * sizeof(float);
  int rc;
  float *dst = static_cast<float *>(r.p);
  if (r.mode) {
    if (!s->conv_tmp && (rc = s->alloc(&s->conv_tmp, cells))) return rc;
    dst = s->conv_tmp;
  }
  rc = s->cuda(cudaMemcpyAsync(dst, src, n, where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               s->stream), "set_field");
  if (rc) return rc;
  if (r.mode) launch_f32_to_h16(s->conv_tmp, static_cast<uint16_t *>(r.p), (long long)cells, r.mode, s->stream);
  return s->sync("set_field");
}
int dcg_get_dense(dcg_sim *s, int32_t field, float *dst, int32_t where) {
  if (bad(s) || !dst) return DCG_E_INVALID;
  if (s->mode == DCG_MODE_UNIFORM) return dcg_get_field(s, field, dst, where);
  const FieldRef r = field_ref(s, field);
  if (!r.p) return s->fail(DCG_E_NOT_FOUND, "no such field");
  const size_t n = (size_t)s->P.gx * s->P.gy * s->P.gz;
  int rc;
  if (!s->dense_tmp && (rc = s->alloc(&s->dense_tmp, n))) return rc;
  launch_fields_to_dense(s->D, r.p, r.mode, s->dense_tmp, s->stream);
  rc = s->cuda(cudaMemcpyAsync(dst, s->dense_tmp, n * 4,
                               where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s->stream),
               "get_dense");
  if (rc) return rc;
  return s->sync("get_dense");
}

int dcg_get_topology(dcg_sim *s, int32_t *pos, uint32_t *parent, uint32_t *child, uint8_t *flags, int64_t *load,
                     int64_t *move_limit) {
  if (bad(s) || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  const long long B = s->D.g.B;
  int rc = 0;
  auto cp = [&](void *dst, const void *src, size_t n) {
    if (dst && !rc) rc = s->cuda(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, s->stream), "get_topology");
  };
  cp(pos, s->D.pos, B * sizeof(int4));
  cp(parent, s->D.parent, B * 4);
  cp(child, s->D.child, 8 * B * 4);
  cp(flags, s->D.flags, B);
  cp(load, s->D.load, s->D.g.levels * 8);
  cp(move_limit, s->D.move_limit, s->D.g.levels * 8);
  if (rc) return rc;
  return s->sync("get_topology");
}
int dcg_set_topology(dcg_sim *s, const int32_t *pos, const uint32_t *parent, const uint32_t *child,
                     const int64_t *load, const int64_t *move_limit) {
  if (bad(s) || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  const long long B = s->D.g.B;
  int rc = 0;
  auto cp = [&](void *dst, const void *src, size_t n) {
    if (src && !rc) rc = s->cuda(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, s->stream), "set_topology");
  };
  cp(s->D.pos, pos, B * sizeof(int4));
  cp(s->D.parent, parent, B * 4);
  cp(s->D.child, child, 8 * B * 4);
  cp(s->D.load, load, s->D.g.levels * 8);
  cp(s->D.move_limit, move_limit, s->D.g.levels * 8);
  if (rc) return rc;
  cudaMemsetAsync(s->D.flags, 0, B, s->stream);
  cudaMemsetAsync(s->D.nbr, 0xff, (size_t)27 * B * 4, s->stream);
  launch_build_nbr(s->D, false, s->stream);
  return s->sync("set_topology");
}
int dcg_get_apron(dcg_sim *s, int64_t *dst) {
  if (bad(s) || !dst || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  const long long B = s->D.g.B;
  int rc;
  if (!s->apron_tmp && (rc = s->alloc(&s->apron_tmp, 216 * B))) return rc;
  launch_apron_table(s->D, s->apron_tmp, s->stream);
  if ((rc = s->cuda(cudaMemcpyAsync(dst, s->apron_tmp, 216 * B * 8, cudaMemcpyDeviceToHost, s->stream), "apron")))
    return rc;
  return s->sync("get_apron");
}
int dcg_get_last_adapt(dcg_sim *s, int64_t *moves, int64_t *n_moves, int64_t *refines, int64_t *n_refines) {
  if (bad(s) || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  long long ctr[C_COUNT];
  int rc;
  if ((rc = s->cuda(cudaMemcpyAsync(ctr, s->D.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, s->stream), "ctr"))) return rc;
  if ((rc = s->sync("ctr"))) return rc;
  const long long nm = ctr[C_MOVES], nr = ctr[C_REFINES];
  if (n_moves) *n_moves = nm;
  if (n_refines) *n_refines = nr;
  std::vector<uint32_t> tmp;
  if (moves && nm > 0) {
    tmp.resize(2 * nm);
    if ((rc = s->cuda(cudaMemcpy(tmp.data(), s->D.moves, 8 * nm, cudaMemcpyDeviceToHost), "moves"))) return rc;
    for (long long i = 0; i < 2 * nm; i++) moves[i] = tmp[i];
  }
  if (refines && nr > 0) {
    tmp.resize(2 * nr);
    if ((rc = s->cuda(cudaMemcpy(tmp.data(), s->D.refines, 8 * nr, cudaMemcpyDeviceToHost), "refines"))) return rc;
    for (long long i = 0; i < 2 * nr; i++) refines[i] = tmp[i];
  }
  return DCG_OK;
}

int dcg_get_stats(dcg_sim *s, dcg_stats *st) {
  if (bad(s) || !st) return DCG_E_INVALID;
  std::memset(st, 0, sizeof(*st));
  st->steps = s->steps;
  int rc;
  double red[32];
  if (s->mode == DCG_MODE_ADAPTIVE) {
    launch_stats(s->D, s->stream);
    long long ctr[C_COUNT], load[MAXL];
    uint32_t e = 0;
    if ((rc = s->cuda(cudaMemcpyAsync(red, s->D.red, sizeof(red), cudaMemcpyDeviceToHost, s->stream), "stats"))) return rc;
    if ((rc = s->cuda(cudaMemcpyAsync(ctr, s->D.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, s->stream), "stats"))) return rc;
    if ((rc = s->cuda(cudaMemcpyAsync(load, s->D.load, sizeof(load), cudaMemcpyDeviceToHost, s->stream), "stats"))) return rc;
    if ((rc = s->cuda(cudaMemcpyAsync(&e, s->D.err, 4, cudaMemcpyDeviceToHost, s->stream), "stats"))) return rc;
    if ((rc = s->sync("stats"))) return rc;
    st->residual = red[0];
    st->mass = red[1];
    for (int l = 0; l < s->D.g.levels; l++) {
      st->load[l] = load[l];
      st->leaf_cells[l] = (int64_t)red[2 + l];
      st->active_cells += st->leaf_cells[l];
    }
    st->moved_blocks = ctr[C_MOVES];
    st->refined_subblocks = ctr[C_REFINES];
    st->device_error = e;
  } else {
    launch_u_stats(s->U, s->stream);
    if ((rc = s->cuda(cudaMemcpyAsync(red, s->U.red, sizeof(red), cudaMemcpyDeviceToHost, s->stream), "stats"))) return rc;
    if ((rc = s->sync("stats"))) return rc;
    st->mass = red[1];
    st->leaf_cells[0] = s->U.nc;
    st->active_cells = s->U.nc;
  }
  return DCG_OK;
}

// Not part of the reference interface: lets tests and benchmarks switch the
// CUDA-graph replay of dcg_step off (1 = on, the default).
int dcg_set_graphs(dcg_sim *s, int32_t on) {
  if (bad(s)) return DCG_E_INVALID;
  s->use_graphs = on != 0;
  return DCG_OK;
}

int dcg_time_kernel(dcg_sim *s, int32_t which, int32_t level, int32_t reps, float *avg_ms, double *bytes) {
  if (bad(s) || !avg_ms || reps <= 0 || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  if (level < 0 || level >= s->D.g.levels) return s->fail(DCG_E_INVALID, "no such level");
  long long load[MAXL];
  int rc;
  if ((rc = s->cuda(cudaMemcpyAsync(load, s->D.load, sizeof(load), cudaMemcpyDeviceToHost, s->stream), "load")))
    return rc;
  if ((rc = s->sync("time_kernel"))) return rc;
  long long alloc = 0;
  for (int l = 0; l < s->D.g.levels; l++) alloc += load[l];
  const double cells_level = 64.0 * (double)load[level], cells_all = 64.0 * (double)alloc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto launch = [&](int i) {
    switch (which) {
      case 0:
        if (i & 1) launch_jacobi(s->D, level, s->D.pt, s->D.p, s->stream);
        else launch_jacobi(s->D, level, s->D.p, s->D.pt, s->stream);
        break;
      case 1: launch_advect_velocity(s->D, s->stream); break;
      case 2: launch_advect_scalars(s->D, s->stream); break;
      case 4: launch_level_solve(s->D, level, 0, s->P.jacobi_iters, s->ls_grid, s->ls_epoch, s->stream); break;
      default: launch_divergence(s->D, s->stream); break;
    }
  };
  if (which == 4 && s->ls_grid <= 0) return s->fail(DCG_E_INVALID, "no cooperative level solve on this device");
  launch(0);  // warm
  cudaEventRecord(e0, s->stream);
  for (int i = 0; i < reps; i++) launch(i);
  cudaEventRecord(e1, s->stream);
  rc = s->sync("time_kernel");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  *avg_ms = ms / (float)reps;
  if (bytes) {
    // algorithmic bytes: each field read once and written once per launch
    const int nq = s->P.n_scalars;
    switch (which) {
      case 0: *bytes = 12.0 * cells_level; break;                  // p r, div r, p~ w
      case 1: *bytes = 24.0 * cells_all; break;                    // v r, v w
      case 2: *bytes = (12.0 + 8.0 * nq) * cells_all; break;       // v r, q r/w
      case 4: *bytes = 12.0 * cells_level * s->P.jacobi_iters; break;  // per sweep: p r, div r, p~ w
      default: *bytes = 16.0 * cells_all; break;                   // v r, div w
    }
  }
  return DCG_OK;
}

int dcg_launches_per_step(dcg_sim *s, int64_t *n) {
  if (bad(s) || !n) return DCG_E_INVALID;
  *n = s->kernels_per_step;
  return DCG_OK;
}

size_t dcg_sizeof_params(void) { return sizeof(dcg_params); }
size_t dcg_sizeof_info(void) { return sizeof(dcg_info); }
size_t dcg_sizeof_stats(void) { return sizeof(dcg_stats); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Dense read-out without device allocation.
//
// dcg_get_dense stages the resampled volume in a device buffer that it
// cudaMallocs on its first call. Some callers cannot allocate at that point:
// code running while a stream is being captured into a CUDA graph (an
// allocation there breaks or invalidates the capture), hosts that hand the
// library a fixed device-memory budget up front, and real-time loops that must
// not hit the allocator's synchronisation. dcg_get_dense_noalloc runs the same
// resampling kernel but stages through the fixed array below, so the call
// itself allocates nothing.
//
// The array is a file-scope __device__ variable: every GPU that loads this
// library holds its 4 MiB until the process exits. In host code its name is
// only a host-side shadow, not a device address, so the kernel is given the
// address that cudaGetSymbolAddress returns, looked up once per device with
// that device current.
namespace {
constexpr size_t kDenseScratchCells = size_t(1) << 20;  // 4 MiB of float
static __device__ __align__(256) float g_dense_scratch[kDenseScratchCells];

std::mutex g_scratch_mu;
float *g_scratch_ptr[64] = {};

int dense_scratch_for_device(int device, float **out, std::string &err) {
  if (device < 0 || device >= 64) {
    err = "device ordinal out of range for the no-allocation scratch";
    return DCG_E_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[device]) {
    int prev = -1;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
    void *p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_dense_scratch);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) {
      err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return DCG_E_CUDA;
    }
    g_scratch_ptr[device] = static_cast<float *>(p);
  }
  *out = g_scratch_ptr[device];
  return DCG_OK;
}
}  // namespace

extern "C" int dcg_get_dense_noalloc(dcg_sim *s, int32_t field, float *dst, int32_t where) {
  if (bad(s) || !dst) return DCG_E_INVALID;
  if (s->mode == DCG_MODE_UNIFORM) return dcg_get_field(s, field, dst, where);  // no staging needed
  const FieldRef src = field_ref(s, field);
  if (!src.p) return s->fail(DCG_E_NOT_FOUND, "no such field");
  const size_t n = (size_t)s->P.gx * s->P.gy * s->P.gz;
  if (n > kDenseScratchCells) {
    char buf[160];
    std::snprintf(buf, sizeof buf,
                  "dense volume of %zu cells exceeds the %zu-cell scratch of dcg_get_dense_noalloc; "
                  "use dcg_get_dense", n, kDenseScratchCells);
    return s->fail(DCG_E_INVALID, buf);
  }
  float *scratch = nullptr;
  int rc = dense_scratch_for_device(s->device, &scratch, s->err);
  if (rc) return rc;
  // The kernel writes every one of the n staged cells, so nothing needs zeroing.
  launch_fields_to_dense(s->D, src.p, src.mode, scratch, s->stream);
  rc = s->cuda(cudaMemcpyAsync(dst, scratch, n * 4,
                               where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s->stream),
               "get_dense_noalloc");
  if (rc) return rc;
  return s->sync("get_dense_noalloc");
}
