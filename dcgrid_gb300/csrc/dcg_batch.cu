// dcg_batch.cu — many independent adaptive simulations stepped together.
//
// The reference runs one simulation per process (its parameters live in one
// global __constant__ block, src/utils/sim_utils.h:5-6). A batch holds n member
// simulations (dcg_sim objects with their own pools) and issues each field
// stage of the step (fluid_simulation_dcgrid.cu:263-346 order) as one launch
// over all members: the members' device descriptors travel in the kernel
// parameters, and a CTA picks its member from the cumulative CTA counts.
// The pressure cascade is one cooperative launch per round over the members'
// concatenated cells of one level; p, p~ and div of all members are slices of
// three batch arenas so the solve addresses them with one base pointer. The
// adaptation (scores, radix sorts, selections, moves, refinements, neighbour
// rebuild, propagation) is likewise one launch per adaptation kernel over all
// members, each member's sorts and counters kept separate. Per-member arithmetic is the
// single simulation's, so results are bit-identical to standalone runs.
#include <chrono>

#include "dcg_sim.h"

struct dcg_batch {
  std::vector<dcg_sim *> m;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<SortScratch> S2;  // members' second sort scratch (block sorts)
  int device = 0, sms = 148;
  std::string err;
  std::vector<void *> allocs;
  size_t bytes = 0;
  float *p_arena = nullptr, *pt_arena = nullptr, *div_arena = nullptr;
  // FP64 defect correction (every member the same number of passes): the
  // correction e, its ping-pong plane and the residual, as arenas laid out like
  // p; the members' norms, 2 (passes + 1) doubles each
  int dpass = 0;
  float *e_arena = nullptr, *et_arena = nullptr, *rr_arena = nullptr;
  double *dnorm_arena = nullptr;
  // planes the cascade runs on: 0 = p, p~, div; 1 = e, e~, r (the correction)
  int planes = 0;
  uint32_t *binfo = nullptr;  // block descriptions of a cascade round, BI_WORDS words per block
  uint32_t *bar = nullptr, *errw = nullptr;
  // concurrent cascades (solve_barrier bit 2): members with two different level
  // counts solved by two cooperative launch chains on parallel graph branches,
  // each with its own barrier words and block-description table
  std::vector<int> lgroup[2];
  uint32_t *bar2 = nullptr, *binfo2 = nullptr;
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::vector<unsigned long long> arena_off;
  unsigned long long arena_cells = 0;
  float *emis_arena = nullptr;  // members' emission maps, consecutive in member order
  size_t emis_floats = 0;
  int maxtop = 0, iters = 0;
  dcg_tuning tune{};
  int solve_grid = 0;
  std::map<int, cudaGraphExec_t> graphs;
  long long kernels_per_step = 0;
  // the members' statistics: one device record per member, read back with
  // one copy into pinned memory
  StatRecord *stage = nullptr, *stage_dev = nullptr;

  int fail(int code, const std::string &msg) {
    err = msg;
    return code;
  }
  int cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return DCG_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
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
  void drop_graphs() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
  }
  ~dcg_batch() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graphs();
    for (dcg_sim *s : m) delete s;
    for (void *p : allocs) cudaFree(p);
    if (stage) cudaFreeHost(stage);
    if (aux) cudaStreamDestroy(aux);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }

  int n() const { return (int)m.size(); }
  int groups() const { return (n() + BMAX - 1) / BMAX; }

  int set_solve_config() {
    if (tune.solve_barrier < 0 || tune.solve_barrier > 7)
      return fail(DCG_E_INVALID, "solve_barrier must be 0..7 (bit 0 two-level barrier, bit 1 coarsest-aligned rounds, "
                                 "bit 2 concurrent cascades of the two level counts)");
    if (!solve_variant_valid(tune.solve_cache))
      return fail(DCG_E_INVALID, "solve_cache must be 0, 3, 4, 8 or a pipelined variant 16, 18, 19, 32, 34, 35, 64, 66, 83");
    for (int k = 0; k < 4; k++)
      if (tune.tile[k] != 1 && tune.tile[k] != 2 && tune.tile[k] != 4 && tune.tile[k] != 8)
        return fail(DCG_E_INVALID, "tiles must be 1 (staged), 2, 4 or 8 blocks");
    solve_grid = batch_solve_grid(sms, tune.solve_cache, tune.solve_ctas_per_sm);
    if (solve_grid <= 0) return fail(DCG_E_CUDA, "cooperative level solve cannot be resident");
    for (int r = 0; r < 4; r++) {
      if (tune.round_ctas_per_sm[r] == 0) continue;
      const int c = tune.round_cache[r];
      if (!solve_variant_valid(c) || (tune.round_barrier[r] != 0 && tune.round_barrier[r] != 1))
        return fail(DCG_E_INVALID, "round schedule: a valid solve variant and barrier 0 or 1");
      if (batch_solve_grid(sms, c, tune.round_ctas_per_sm[r]) <= 0)
        return fail(DCG_E_CUDA, "round schedule cannot be resident");
    }
    return DCG_OK;
  }

  // ------------------------------------------------------------ stage launches
  // the members a stage launch covers: all, or the listed ones
  std::vector<int> all_members() const {
    std::vector<int> v(n());
    for (int i = 0; i < n(); i++) v[i] = i;
    return v;
  }
  void cells(int stage) { cells(stage, all_members(), stream); }
  void cells(int stage, const std::vector<int> &mem, cudaStream_t st) {
    for (size_t g = 0; g < mem.size(); g += BMAX) {
      CellBatch P{};
      P.n = (int)std::min<size_t>(BMAX, mem.size() - g);
      for (int i = 0; i < P.n; i++) P.d[i] = m[mem[g + i]]->D;
      launch_cells_batch(stage, P, stage == 5 ? 1 : tune.tile[stage], st, tune.persistent != 0);
    }
  }
  // field: 0 velocity, 1 scalars, 2 divergence, 3 velocity and scalars
  void restrict_fields(int field) { restrict_fields(field, all_members(), stream); }
  void restrict_fields(int field, const std::vector<int> &mem, cudaStream_t st) {
    int maxl = 0;
    for (int i : mem) maxl = std::max(maxl, m[i]->D.g.levels);
    for (int level = 0; level < maxl - 1; level++)
      for (size_t g = 0; g < mem.size(); g += BMAX) {
        RestrictBatch P{};
        P.n = (int)std::min<size_t>(BMAX, mem.size() - g);
        P.level = level;
        for (int i = 0; i < P.n; i++) {
          const dcg_sim *s = m[mem[g + i]];
          P.d[i] = s->D;
          FieldList &fl = P.fl[i];
          if (field == 0 || field == 3) {
            fl.n = 3;
            for (int d = 0; d < 3; d++) fl.f[d] = s->D.v[d];
          }
          if (field == 1 || field == 3) {
            const int o = fl.n;
            fl.n += s->P.n_scalars;
            for (int k = 0; k < s->P.n_scalars; k++) {
              fl.f[o + k] = s->D.g.mixed ? static_cast<void *>(s->D.qh[k]) : static_cast<void *>(s->D.q[k]);
              fl.mode[o + k] = s->D.g.mixed;
            }
          }
          if (field == 2) {
            fl.n = 1;
            fl.f[0] = s->D.div;
          }
        }
        launch_restrict_batch(P, st);
      }
  }
  // the arenas of the planes the cascade runs on; with the correction planes,
  // the members' descriptors name them too (the prolongation and the cached
  // alpha * div read them through the descriptor)
  void bind_planes(SolveBatch &P) const {
    if (planes == 0) {
      P.p = p_arena;
      P.pt = pt_arena;
      P.div = div_arena;
      return;
    }
    P.p = e_arena;
    P.pt = et_arena;
    P.div = rr_arena;
    for (int i = 0; i < P.n; i++) {
      P.d[i].p = P.d[i].e;
      P.d[i].pt = P.d[i].et;
      P.d[i].div = P.d[i].rr;
    }
  }
  // FP64 defect correction after the cascade (dcg_sim::defect_correct for
  // every member): per pass the FP64 residual and norms, the cascade on the
  // residual into e, and p += e; a last residual measures the result
  void defect_correct() {
    cudaMemsetAsync(dnorm_arena, 0, sizeof(double) * 2 * (dpass + 1) * n(), stream);
    for (int k = 0; k <= dpass; k++) {
      for (int g = 0; g < groups(); g++) {
        CellBatch P{};
        P.n = std::min(BMAX, n() - g * BMAX);
        for (int i = 0; i < P.n; i++) P.d[i] = m[g * BMAX + i]->D;
        P.arg = k;
        launch_cells_batch(6, P, 1, stream);  // FP64 residual of pass k
      }
      if (k == dpass) break;
      cudaMemsetAsync(e_arena, 0, (size_t)arena_cells * sizeof(float), stream);
      planes = 1;
      solve_tuned();
      planes = 0;
      for (int g = 0; g < groups(); g++) {
        CellBatch P{};
        P.n = std::min(BMAX, n() - g * BMAX);
        for (int i = 0; i < P.n; i++) P.d[i] = m[g * BMAX + i]->D;
        launch_add_correction_batch(P, stream);
      }
    }
  }
  // the cascade with the tuned schedule of each round
  bool can_split() const { return n() <= BMAX && !lgroup[0].empty() && !lgroup[1].empty() && aux; }
  // one member group's whole cascade (all its members have the same level count)
  void solve_group(int gi, int grid, int cache, int tree, cudaStream_t st) {
    const std::vector<int> &mem = lgroup[gi];
    const int top = m[mem[0]]->D.g.levels - 1;
    for (int round = 0; round <= top; round++) {
      SolveBatch P{};
      P.n = (int)mem.size();
      P.maxtop = top;
      P.prolong = 1;
      P.binfo = gi ? binfo2 : binfo;
      P.bar = gi ? bar2 : bar;
      P.err = errw;
      for (int i = 0; i < P.n; i++) {
        P.d[i] = m[mem[i]]->D;
        P.arena[i] = arena_off[mem[i]];
      }
      bind_planes(P);
      launch_level_solve_batch(P, round, iters, grid, cache, tree & 1, st);
    }
  }
  void solve_split(int grid, int cache, int tree) {
    cudaEventRecord(ev_fork, stream);
    cudaStreamWaitEvent(aux, ev_fork, 0);
    solve_group(0, grid, cache, tree, stream);
    solve_group(1, grid, cache, tree, aux);
    cudaEventRecord(ev_join, aux);
    cudaStreamWaitEvent(stream, ev_join, 0);
  }
  void solve_tuned() {
    if ((tune.solve_barrier & 4) && can_split()) {
      solve_split(solve_grid, tune.solve_cache, tune.solve_barrier);
      return;
    }
    for (int round = 0; round <= maxtop; round++) {
      if (round < 4 && tune.round_ctas_per_sm[round] != 0)
        solve_round(round, batch_solve_grid(sms, tune.round_cache[round], tune.round_ctas_per_sm[round]),
                    tune.round_cache[round], tune.round_barrier[round]);
      else
        solve_round(round, solve_grid, tune.solve_cache, tune.solve_barrier & 1);
    }
  }
  void solve(int grid, int cache, int tree) {
    if ((tune.solve_barrier & 4) && can_split()) {
      solve_split(grid, cache, tree);
      return;
    }
    for (int round = 0; round <= maxtop; round++) solve_round(round, grid, cache, tree);
  }
  // tree: two-level barrier; the round alignment comes from tune.solve_barrier's bit 1
  void solve_round(int round, int grid, int cache, int tree) {
    tree = (tree & 1) | (tune.solve_barrier & 2);
    {
      for (int g = 0; g < groups(); g++) {
        SolveBatch P{};
        P.n = std::min(BMAX, n() - g * BMAX);
        P.maxtop = maxtop;
        P.prolong = 1;
        P.binfo = binfo;
        P.bar = bar;
        P.err = errw;
        for (int i = 0; i < P.n; i++) {
          P.d[i] = m[g * BMAX + i]->D;
          P.arena[i] = arena_off[g * BMAX + i];
        }
        bind_planes(P);
        launch_level_solve_batch(P, round, iters, grid, cache, tree, stream);  // bit 1: alignment
      }
    }
  }
  void flip_v() {
    for (dcg_sim *s : m) {
      s->vpar ^= 1;
      s->bind_parity();
    }
  }
  void flip_q() {
    for (dcg_sim *s : m) {
      s->qpar ^= 1;
      s->bind_parity();
    }
  }
  // every member's adaptation, one launch per adaptation kernel and group
  void adapt() {
    for (int g = 0; g < groups(); g++) {
      AdaptMember A[BMAX];
      const int k = std::min(BMAX, n() - g * BMAX);
      for (int i = 0; i < k; i++) {
        const dcg_sim *s = m[g * BMAX + i];
        A[i] = AdaptMember{s->D, s->S, S2[g * BMAX + i], s->keys, s->vals, s->keys2, s->vals2};
      }
      launch_adapt_batch(A, k, sms, stream);
    }
  }
  // Simulation::updateSimulation (simulation.cpp:104-112) for every member
  // the pressure application and the scalar advection run as one staged pass
  // when both stages are tuned to their staged forms
  bool fused() const { return tune.tile[1] == 1 && tune.tile[3] == 1; }
  void apply_advect() {
    if (fused()) {
      cells(5);  // apply pressure + advect scalars (+ sources, emission)
      flip_q();
      restrict_fields(3);
    } else {
      cells(3);  // apply pressure
      restrict_fields(0);
      cells(1);  // advect scalars (+ sources, emission)
      flip_q();
      restrict_fields(1);
    }
  }
  // With rounds aligned at the coarsest levels, the members with fewer levels
  // finish their cascade a round early. Their pressure application, scalar
  // advection and restrictions then run on the second stream (a parallel
  // graph branch) while the last rounds relax the other members: the
  // stages read and write only their own members' planes, and the late
  // rounds, small and bound by their grid barriers, leave most of the GPU free.
  bool overlapped() const {
    return dpass == 0 && fused() && can_split() && (tune.solve_barrier & 2) && !(tune.solve_barrier & 4);
  }
  void apply_advect_members(const std::vector<int> &mem, cudaStream_t st) {
    cells(5, mem, st);  // apply pressure + advect scalars (+ sources, emission)
    for (int i : mem) {
      m[i]->qpar ^= 1;
      m[i]->bind_parity();
    }
    restrict_fields(3, mem, st);
  }
  void solve_apply_overlapped() {
    const int ga = m[lgroup[0][0]]->D.g.levels < m[lgroup[1][0]]->D.g.levels ? 0 : 1;  // fewer levels
    const int last = m[lgroup[ga][0]]->D.g.levels - 1;  // its last round
    for (int round = 0; round <= maxtop; round++) {
      if (round < 4 && tune.round_ctas_per_sm[round] != 0)
        solve_round(round, batch_solve_grid(sms, tune.round_cache[round], tune.round_ctas_per_sm[round]),
                    tune.round_cache[round], tune.round_barrier[round]);
      else
        solve_round(round, solve_grid, tune.solve_cache, tune.solve_barrier & 1);
      if (round == last) {
        cudaEventRecord(ev_fork, stream);
        cudaStreamWaitEvent(aux, ev_fork, 0);
        apply_advect_members(lgroup[ga], aux);
        cudaEventRecord(ev_join, aux);
      }
    }
    apply_advect_members(lgroup[1 - ga], stream);
    cudaStreamWaitEvent(stream, ev_join, 0);
  }
  void step_once() {
    cells(0);  // advect velocity (+ buoyancy)
    flip_v();
    restrict_fields(0);
    adapt();
    cells(2);  // divergence
    restrict_fields(2);
    if (overlapped()) {
      solve_apply_overlapped();
      return;
    }
    solve_tuned();
    if (dpass > 0) defect_correct();
    apply_advect();
  }

  // One step as step_once() without the graph, with CUDA events between the
  // stages and the pressure application and scalar advection as separate
  // passes: ms[0] velocity advection (+ its restriction), [1] adaptation,
  // [2] divergence (+ restriction), [3] pressure cascade (+ defect
  // correction), [4] pressure application (+ restriction), [5] scalar
  // advection (+ restriction), [6] the whole step.
  int profile_step(float *ms) {
    cudaEvent_t ev[7];
    for (auto &e : ev) cudaEventCreate(&e);
    cudaEventRecord(ev[0], stream);
    cells(0);
    flip_v();
    restrict_fields(0);
    cudaEventRecord(ev[1], stream);
    adapt();
    cudaEventRecord(ev[2], stream);
    cells(2);
    restrict_fields(2);
    cudaEventRecord(ev[3], stream);
    solve_tuned();
    if (dpass > 0) defect_correct();
    cudaEventRecord(ev[4], stream);
    cells(3);
    restrict_fields(0);
    cudaEventRecord(ev[5], stream);
    cells(1);
    flip_q();
    restrict_fields(1);
    cudaEventRecord(ev[6], stream);
    int rc = cuda(cudaEventSynchronize(ev[6]), "profile step");
    for (int k = 0; k < 6 && !rc; k++) cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
    if (!rc) cudaEventElapsedTime(&ms[6], ev[0], ev[6]);
    for (auto &e : ev) cudaEventDestroy(e);
    for (dcg_sim *s : m) s->steps++;
    if (rc) return rc;
    return cuda(cudaGetLastError(), "profile step");
  }

  int step(int count) {
    for (int i = 0; i < count; i++) {
      const int key = m[0]->vpar * 2 + m[0]->qpar;
      auto it = graphs.find(key);
      int rc;
      if (it == graphs.end()) {
        cudaGraph_t g = nullptr;
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
        rc = cuda(cudaGraphInstantiate(&ge, g, 0), "instantiate");
        cudaGraphDestroy(g);
        if (rc) return rc;
        graphs[key] = ge;
        // step_once() advanced the members' parities while capturing
        if ((rc = cuda(cudaGraphLaunch(ge, stream), "graph launch"))) return rc;
      } else {
        if ((rc = cuda(cudaGraphLaunch(it->second, stream), "graph launch"))) return rc;
        flip_v();
        flip_q();
      }
      for (dcg_sim *s : m) s->steps++;
    }
    return cuda(cudaGetLastError(), "batch step");
  }

  int reset() {
    int rc;
    if ((rc = cuda(cudaStreamSynchronize(stream), "sync"))) return rc;
    cudaMemsetAsync(bar, 0, 4 * (64 + 32 * 18), stream);
    if (bar2) cudaMemsetAsync(bar2, 0, 4 * (64 + 32 * 18), stream);
    cudaMemsetAsync(errw, 0, 4, stream);
    for (dcg_sim *s : m)
      if ((rc = s->reset_adaptive())) return fail(rc, "member reset: " + s->err);
    return cuda(cudaStreamSynchronize(stream), "reset");
  }

  int sync() {
    int rc;
    if ((rc = cuda(cudaStreamSynchronize(stream), "sync"))) return rc;
    if ((rc = cuda(cudaGetLastError(), "sync"))) return rc;
    uint32_t e = 0;
    if ((rc = cuda(cudaMemcpy(&e, errw, 4, cudaMemcpyDeviceToHost), "err word"))) return rc;
    if (e) {
      char buf[64];
      std::snprintf(buf, sizeof buf, "batch device error word 0x%x", e);
      return fail(DCG_E_DEVICE, buf);
    }
    // a non-finite value (DCG_E_NAN) is reported only when no member has a
    // more serious error
    int nan_member = -1;
    for (int i = 0; i < n(); i++) {
      if ((rc = cuda(cudaMemcpy(&e, m[i]->D.err, 4, cudaMemcpyDeviceToHost), "err word"))) return rc;
      if (e == DCG_DEVERR_NAN) {
        if (nan_member < 0) nan_member = i;
      } else if (e) {
        char buf[80];
        std::snprintf(buf, sizeof buf, "member %d device error word 0x%x", i, e);
        return fail(DCG_E_DEVICE, buf);
      }
    }
    if (nan_member >= 0)
      return fail(DCG_E_NAN, "member " + std::to_string(nan_member) + ": a non-finite value in a leaf cell");
    return DCG_OK;
  }

  // CUDA-event time of fn() averaged over reps (one warm call first)
  template <class F> float time_ms(int reps, F fn) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fn();
    cudaEventRecord(e0, stream);
    for (int r = 0; r < reps; r++) fn();
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / (float)reps;
  }

  int autotune(int spinup, int reps, dcg_tuning *out) {
    int rc;
    if ((rc = reset())) return rc;
    if ((rc = step(spinup))) return rc;
    if ((rc = sync())) return rc;
    // cell stages: every tile of each stage, launched one CTA per block or
    // persistent; the launch form that gives the lower total is kept. Tile 1:
    // one warp per block through shared tiles (staged)
    const int tiles[4] = {1, 2, 4, 8};
    dcg_tuning best = tune;
    float total[2] = {0.f, 0.f};
    int tile_of[2][4];
    float ms_of[2][4];
    for (int pers = 0; pers < 2; pers++) {
      tune.persistent = pers;
      for (int stage = 0; stage < 4; stage++) {
        float best_ms = 1e30f;
        for (int tile : tiles) {
          tune.tile[stage] = tile;
          const float ms = time_ms(reps, [&] { cells(stage); });
          if (ms < best_ms) {
            best_ms = ms;
            tile_of[pers][stage] = tile;
          }
        }
        ms_of[pers][stage] = best_ms;
        total[pers] += best_ms;
        tune.tile[stage] = tile_of[pers][stage];
      }
    }
    const int pick = total[1] < total[0] ? 1 : 0;
    best.persistent = pick;
    tune.persistent = pick;
    for (int stage = 0; stage < 4; stage++) {
      best.tile[stage] = tune.tile[stage] = tile_of[pick][stage];
      best.cells_ms[stage] = ms_of[pick][stage];
    }
    // level solve: cache depth x CTAs per SM x barrier kind
    float best_solve = 1e30f;
    for (int cache : {0, 3, 4, 8, 16, 18, 19, 32, 34, 35, 64, 66, 83}) {
      const int occ = batch_solve_grid(sms, cache, 0) / std::max(1, sms);
      for (int k = 1; k <= occ; k++)
        for (int tb = 0; tb < 8; tb++) {  // bit 0: two-level barrier; bit 1: coarsest-aligned rounds;
                                          // bit 2: concurrent cascades per level count
          if ((tb & 4) && (!can_split() || (tb & 2))) continue;
          tune.solve_barrier = tb;
          const int grid = batch_solve_grid(sms, cache, k);
          const float ms = time_ms(reps, [&] { solve(grid, cache, tb & 1); });
          if (ms < best_solve) {
            best_solve = ms;
            best.solve_cache = cache;
            best.solve_ctas_per_sm = k;
            best.solve_barrier = tb;
          }
        }
    }
    tune.solve_barrier = best.solve_barrier;  // the per-round schedules below use its alignment
    // each round of the first four on its own: the best schedule if it beats
    // the whole-cascade choice for that round (not with concurrent cascades)
    for (int r = 0; r < 4 && r <= maxtop && !(best.solve_barrier & 4); r++) {
      const float base = time_ms(reps, [&] {
        solve_round(r, batch_solve_grid(sms, best.solve_cache, best.solve_ctas_per_sm), best.solve_cache,
                    best.solve_barrier);
      });
      float bms = base;
      best.round_ctas_per_sm[r] = 0;
      for (int cache : {0, 3, 4, 8, 16, 18, 19, 32, 34, 35, 64, 66, 83}) {
        const int occ = batch_solve_grid(sms, cache, 0) / std::max(1, sms);
        std::vector<int> ks = {-8, -4, -2};  // k < 0: one CTA per -k SMs (small rounds)
        for (int k = 1; k <= occ; k++) ks.push_back(k);
        for (int k : ks)
          for (int tree = 0; tree < 2; tree++) {
            const int grid = batch_solve_grid(sms, cache, k);
            const float ms = time_ms(reps, [&] { solve_round(r, grid, cache, tree); });
            if (ms < 0.97f * bms) {
              bms = ms;
              best.round_ctas_per_sm[r] = (int16_t)k;
              best.round_cache[r] = (int8_t)cache;
              best.round_barrier[r] = (int8_t)tree;
            }
          }
      }
      best_solve += bms - base;
    }
    best.solve_ms = best_solve;
    if ((rc = sync())) return rc;
    tune = best;
    if ((rc = set_solve_config())) return rc;
    drop_graphs();
    if ((rc = reset())) return rc;
    if (out) *out = tune;
    return DCG_OK;
  }

  // every member's statistics with one launch per group and one synchronisation
  int get_stats(dcg_stats *out) {
    int rc;
    if (!stage && (rc = cuda(cudaMallocHost(&stage, sizeof(StatRecord) * n()), "stats staging"))) return rc;
    if (!stage_dev && (rc = alloc(&stage_dev, n()))) return rc;
    for (int g = 0; g < groups(); g++) {
      CellBatch P{};
      P.n = std::min(BMAX, n() - g * BMAX);
      for (int i = 0; i < P.n; i++) P.d[i] = m[g * BMAX + i]->D;
      launch_stats_zero(P, stream);
      launch_cells_batch(4, P, 1, stream, true);  // staged statistics
      launch_stats_gather(P, stage_dev + g * BMAX, stream);
    }
    cudaMemcpyAsync(stage, stage_dev, sizeof(StatRecord) * n(), cudaMemcpyDeviceToHost, stream);
    if ((rc = cuda(cudaStreamSynchronize(stream), "stats"))) return rc;
    for (int i = 0; i < n(); i++) {
      dcg_stats &st = out[i];
      std::memset(&st, 0, sizeof st);
      const StatRecord &x = stage[i];
      st.steps = m[i]->steps;
      st.residual = x.red[0];
      st.mass = x.red[1];
      for (int l = 0; l < m[i]->D.g.levels; l++) {
        st.load[l] = x.load[l];
        st.leaf_cells[l] = (int64_t)x.red[2 + l];
        st.active_cells += st.leaf_cells[l];
      }
      st.moved_blocks = x.ctr[C_MOVES];
      st.refined_subblocks = x.ctr[C_REFINES];
      st.device_error = x.err;
      if (dpass > 0) {
        auto rel = [](double r2, double b2) { return b2 > 0 ? std::sqrt(r2 / b2) : 0.0; };
        st.defect_rel_residual[0] = rel(x.dn[0], x.dn[1]);
        st.defect_rel_residual[1] = rel(x.dn[2], x.dn[3]);
      }
    }
    // the statistics are filled either way; the status reports a non-finite value
    for (int i = 0; i < n(); i++)
      if (out[i].device_error & DCG_DEVERR_NAN)
        return fail(DCG_E_NAN, "member " + std::to_string(i) + ": a non-finite value in a leaf cell");
    return DCG_OK;
  }

  int time_solve(int reps, float *avg_ms, double *bytes_out) {
    int rc;
    if ((rc = sync())) return rc;
    double cells_sweeps = 0;
    for (dcg_sim *s : m) {
      long long load[MAXL];
      if ((rc = cuda(cudaMemcpy(load, s->D.load, sizeof(load), cudaMemcpyDeviceToHost), "load"))) return rc;
      for (int l = 0; l < s->D.g.levels; l++) cells_sweeps += 64.0 * (double)load[l] * iters;
    }
    *avg_ms = time_ms(reps, [&] { solve_tuned(); });
    if (bytes_out) *bytes_out = 12.0 * cells_sweeps;
    return sync();
  }
};

static int bad(const dcg_batch *b) { return b == nullptr; }

extern "C" {

int dcg_batch_create(int32_t n, const dcg_params *params, dcg_batch **out) {
  if (!params || !out || n <= 0) return DCG_E_INVALID;
  *out = nullptr;
  dcg_batch *b = new dcg_batch();
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return DCG_E_CUDA;
  }
  b->own_stream = true;
  b->iters = params[0].jacobi_iters;
  b->dpass = params[0].defect_passes;
  // arenas for p and p~: member i's planes start at cell arena_off[i]
  unsigned long long cells = 0;
  for (int i = 0; i < n; i++) {
    if (params[i].jacobi_iters != b->iters) {
      delete b;
      return DCG_E_INVALID;  // one sweep schedule per batch
    }
    if (params[i].max_blocks <= 0 || params[i].max_blocks >= (1ll << 28) || params[i].defect_passes != b->dpass ||
        b->dpass < 0 || b->dpass > 16) {
      delete b;
      return DCG_E_INVALID;  // one defect-correction schedule per batch
    }
    b->arena_off.push_back(cells);
    cells += (unsigned long long)params[i].max_blocks * BV;
  }
  if (cells >= (1ull << 32)) {
    delete b;
    return DCG_E_INVALID;  // arena cells are addressed with 32-bit indices
  }
  b->arena_cells = cells;
  int rc;
  if (b->dpass > 0 &&
      ((rc = b->alloc(&b->e_arena, cells)) || (rc = b->alloc(&b->et_arena, cells)) ||
       (rc = b->alloc(&b->rr_arena, cells)) || (rc = b->alloc(&b->dnorm_arena, 2 * (b->dpass + 1) * (size_t)n)))) {
    delete b;
    return rc;
  }
  if ((rc = b->alloc(&b->p_arena, cells)) || (rc = b->alloc(&b->pt_arena, cells)) ||
      (rc = b->alloc(&b->div_arena, cells)) || (rc = b->alloc(&b->binfo, BI_WORDS * (cells / BV))) ||
      (rc = b->alloc(&b->bar, 64 + 32 * 18)) || (rc = b->alloc(&b->errw, 4))) {
    delete b;
    return rc;
  }
  cudaMemset(b->bar, 0, 4 * (64 + 32 * 18));
  for (int i = 0; i < n; i++)
    if (params[i].emission_n > 0)
      b->emis_floats += (size_t)params[i].emission_n * params[i].emission_n * params[i].emission_n;
  if (b->emis_floats > 0 && (rc = b->alloc(&b->emis_arena, b->emis_floats))) {
    delete b;
    return rc;
  }
  if ((rc = b->alloc(&b->bar2, 64 + 32 * 18)) || (rc = b->alloc(&b->binfo2, BI_WORDS * (cells / BV)))) {
    delete b;
    return rc;
  }
  cudaMemset(b->bar2, 0, 4 * (64 + 32 * 18));
  cudaMemset(b->errw, 0, 4);
  size_t emis_at = 0;
  for (int i = 0; i < n; i++) {
    dcg_sim *s = new dcg_sim();
    s->P = params[i];
    s->mode = DCG_MODE_ADAPTIVE;
    s->device = b->device;
    s->sms = b->sms;
    s->stream = b->stream;
    s->own_stream = false;
    s->batch_member = true;
    s->ext_p = b->p_arena + b->arena_off[i];
    s->ext_pt = b->pt_arena + b->arena_off[i];
    s->ext_div = b->div_arena + b->arena_off[i];
    if (b->dpass > 0) {
      s->ext_rr = b->rr_arena + b->arena_off[i];
      s->ext_e = b->e_arena + b->arena_off[i];
      s->ext_et = b->et_arena + b->arena_off[i];
      s->ext_dnorm = b->dnorm_arena + 2 * (size_t)(b->dpass + 1) * i;
    }
    if (params[i].emission_n > 0) {
      s->ext_emis = b->emis_arena + emis_at;
      emis_at += (size_t)params[i].emission_n * params[i].emission_n * params[i].emission_n;
    }
    b->m.push_back(s);
    if ((rc = s->create_adaptive())) {
      b->err = "member " + std::to_string(i) + ": " + s->err;
      delete b;
      return rc;
    }
    b->maxtop = std::max(b->maxtop, s->D.g.levels - 1);
    SortScratch S2{};
    const long long nb = s->D.g.B, nt = sort_tiles(nb);
    if ((rc = b->alloc(&S2.k1, nb)) || (rc = b->alloc(&S2.v1, nb)) || (rc = b->alloc(&S2.hist, 256 * nt)) ||
        (rc = b->alloc(&S2.totals, 256))) {
      delete b;
      return rc;
    }
    S2.max_n = nb;
    b->S2.push_back(S2);
  }
  // level-count groups for concurrent cascades: exactly two level counts
  {
    int la = -1, lb = -1;
    bool two = true;
    for (int i = 0; i < n; i++) {
      const int L = b->m[i]->D.g.levels;
      if (la < 0 || L == la) la = L;
      else if (lb < 0 || L == lb) lb = L;
      else two = false;
    }
    if (two && lb >= 0) {
      for (int i = 0; i < n; i++) b->lgroup[b->m[i]->D.g.levels == la ? 0 : 1].push_back(i);
      if (cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
          cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        delete b;
        return DCG_E_CUDA;
      }
    }
  }
  for (int k = 0; k < 4; k++) b->tune.tile[k] = 4;
  b->tune.solve_cache = 4;
  b->tune.solve_ctas_per_sm = 0;
  b->tune.solve_barrier = 1;
  if ((rc = b->set_solve_config())) {
    delete b;
    return rc;
  }
  *out = b;
  return DCG_OK;
}

int dcg_batch_destroy(dcg_batch *b) {
  if (bad(b)) return DCG_E_INVALID;
  delete b;
  return DCG_OK;
}
int dcg_batch_reset(dcg_batch *b) { return bad(b) ? DCG_E_INVALID : b->reset(); }
int dcg_batch_step(dcg_batch *b, int32_t n) {
  if (bad(b) || n < 0) return DCG_E_INVALID;
  return b->step(n);
}
int dcg_batch_sync(dcg_batch *b) { return bad(b) ? DCG_E_INVALID : b->sync(); }
int dcg_batch_profile_step(dcg_batch *b, float *stage_ms) {
  if (bad(b) || !stage_ms) return DCG_E_INVALID;
  return b->profile_step(stage_ms);
}
int dcg_batch_member(dcg_batch *b, int32_t i, dcg_sim **out) {
  if (bad(b) || !out || i < 0 || i >= b->n()) return DCG_E_INVALID;
  *out = b->m[i];
  return DCG_OK;
}
int dcg_batch_set_stream(dcg_batch *b, void *cuda_stream) {
  if (bad(b)) return DCG_E_INVALID;
  cudaStreamSynchronize(b->stream);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->own_stream = false;
  b->stream = reinterpret_cast<cudaStream_t>(cuda_stream);
  for (dcg_sim *s : b->m) s->stream = b->stream;
  b->drop_graphs();
  return DCG_OK;
}
int dcg_batch_autotune(dcg_batch *b, int32_t spinup_steps, int32_t reps, dcg_tuning *out) {
  if (bad(b) || spinup_steps < 0 || reps <= 0) return DCG_E_INVALID;
  return b->autotune(spinup_steps, reps, out);
}
int dcg_batch_get_tuning(const dcg_batch *b, dcg_tuning *out) {
  if (bad(b) || !out) return DCG_E_INVALID;
  *out = b->tune;
  return DCG_OK;
}
int dcg_batch_set_tuning(dcg_batch *b, const dcg_tuning *t) {
  if (bad(b) || !t) return DCG_E_INVALID;
  const dcg_tuning before = b->tune;
  b->tune = *t;
  int rc = b->set_solve_config();
  if (rc) {
    b->tune = before;
    b->set_solve_config();
    return rc;
  }
  cudaStreamSynchronize(b->stream);
  b->drop_graphs();
  return DCG_OK;
}
int dcg_batch_get_info(const dcg_batch *b, int32_t *n, int64_t *device_bytes, int64_t *launches_per_step) {
  if (bad(b)) return DCG_E_INVALID;
  if (n) *n = b->n();
  if (device_bytes) {
    size_t t = b->bytes;
    for (const dcg_sim *s : b->m) t += s->bytes;
    *device_bytes = (int64_t)t;
  }
  if (launches_per_step) *launches_per_step = b->kernels_per_step;
  return DCG_OK;
}
int dcg_batch_time_solve(dcg_batch *b, int32_t reps, float *avg_ms, double *bytes) {
  if (bad(b) || reps <= 0 || !avg_ms) return DCG_E_INVALID;
  return b->time_solve(reps, avg_ms, bytes);
}
int dcg_batch_set_emission(dcg_batch *b, const float *maps, int32_t where) {
  if (bad(b) || !maps) return DCG_E_INVALID;
  if (b->emis_floats == 0) return b->fail(DCG_E_INVALID, "no member has an emission map");
  return b->cuda(cudaMemcpyAsync(b->emis_arena, maps, b->emis_floats * 4,
                                 where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream),
                 "batch set_emission");
}
int dcg_batch_get_stats(dcg_batch *b, dcg_stats *out) {
  if (bad(b) || !out) return DCG_E_INVALID;
  return b->get_stats(out);
}
const char *dcg_batch_last_error_string(const dcg_batch *b) { return b ? b->err.c_str() : "null handle"; }
size_t dcg_sizeof_tuning(void) { return sizeof(dcg_tuning); }

}  // extern "C"
