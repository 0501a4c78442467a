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

#include "dcg_sim.h"

static int bad(dcg_sim *s) { return s == nullptr; }
// members of a batch are stepped, reconfigured and destroyed through the batch
static int member_refused(dcg_sim *s) {
  return s->batch_member ? s->fail(DCG_E_INVALID, "member of a batch: use the dcg_batch_* calls") : DCG_OK;
}

// Status of a nonzero device error word: DCG_E_NAN when the only bit is the
// non-finite-value flag, else DCG_E_DEVICE (a bounded wait gave up, a block
// budget ran out, a lookup failed).
static int device_error_status(uint32_t e) { return e == DCG_DEVERR_NAN ? DCG_E_NAN : DCG_E_DEVICE; }
static std::string device_error_text(uint32_t e) {
  std::string t = "device error word 0x";
  char buf[16];
  std::snprintf(buf, sizeof buf, "%x", e);
  t += buf;
  if (e & DCG_DEVERR_BUDGET) t += ", a refinement found its level full";
  if (e & DCG_DEVERR_LOOKUP) t += ", a block lookup failed";
  if (e & DCG_DEVERR_NAN) t += ", a non-finite value in a leaf cell";
  if (e & DCG_DEVERR_TIMEOUT) t += ", a bounded device-side wait gave up";
  return t;
}

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
  if (member_refused(sim)) return DCG_E_INVALID;
  cudaStreamSynchronize(sim->stream);
  delete sim;
  return DCG_OK;
}

int dcg_reset(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  return s->mode == DCG_MODE_ADAPTIVE ? s->reset_adaptive() : s->reset_uniform();
}

int dcg_set_params(dcg_sim *s, const dcg_params *p) {
  if (bad(s) || !p) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  if (p->gx != s->P.gx || p->gy != s->P.gy || p->gz != s->P.gz || p->levels != s->P.levels ||
      p->max_blocks != s->P.max_blocks || p->n_scalars != s->P.n_scalars || p->precision != s->P.precision ||
      p->ref_compat != s->P.ref_compat || p->defect_passes != s->P.defect_passes)
    return s->fail(DCG_E_INVALID,
                   "geometry, budget, scalars, precision, compat mode and defect passes are fixed at creation");
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
  if (member_refused(*sim)) return DCG_E_INVALID;
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
  if (member_refused(s)) return DCG_E_INVALID;
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
  if (member_refused(s)) return DCG_E_INVALID;
  return s->step(n);
}
int dcg_advect_velocity(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  s->stage_advect_velocity();
  return s->check_launch("advect_velocity");
}
int dcg_adapt(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  s->stage_adapt();
  return s->check_launch("adapt");
}
int dcg_project(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  s->stage_project(false);
  return s->check_launch("project");
}
int dcg_project_local(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  s->stage_project(true);
  return s->check_launch("project_local");
}
int dcg_advect_scalars(dcg_sim *s) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
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
    if (e) return s->fail(device_error_status(e), device_error_text(e));
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

int dcg_set_heightmap(dcg_sim *s, const float *heights, int32_t nx, int32_t nz, int32_t where) {
  if (bad(s)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  if (heights && (nx <= 0 || nz <= 0 || nx > 65536 || nz > 65536 || (long long)nx * nz > (1ll << 27)))
    return s->fail(DCG_E_INVALID, "heightmap: 1 <= nx, nz <= 65536 and nx * nz <= 2^27");
  if (!heights && (nx != 0 || nz != 0)) return s->fail(DCG_E_INVALID, "heightmap: no heights given for nx, nz > 0");
  int rc;
  if ((rc = s->sync("set_heightmap"))) return rc;  // steps in flight may read the old map
  // captured step graphs hold the physics, and with it the map pointer, by value
  for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  if (s->hmap) cudaFree(s->hmap);
  s->hmap = nullptr;
  s->hm_nx = s->hm_nz = 0;
  if (heights) {
    const size_t n = (size_t)nx * nz;
    float *h = nullptr;
    rc = s->cuda(cudaMalloc(&h, n * sizeof(float)), "set_heightmap");
    if (!rc)
      rc = s->cuda(cudaMemcpyAsync(h, heights, n * sizeof(float),
                                   where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   s->stream), "set_heightmap");
    if (rc) {
      if (h) cudaFree(h);
    } else {
      s->hmap = h;
      s->hm_nx = nx;
      s->hm_nz = nz;
    }
  }
  s->fill_phys(s->D.ph);
  s->fill_phys(s->U.ph);
  if (rc) return rc;  // back on the noise terrain
  return s->mode == DCG_MODE_ADAPTIVE ? s->reset_adaptive() : s->reset_uniform();
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
  bool nan_seen = false;
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
    nan_seen = (e & DCG_DEVERR_NAN) != 0;
    if (s->P.defect_passes > 0) {
      const int K = s->P.defect_passes;
      std::vector<double> dn(2 * (K + 1));
      if ((rc = s->cuda(cudaMemcpy(dn.data(), s->D.dnorm, dn.size() * 8, cudaMemcpyDeviceToHost), "stats"))) return rc;
      auto rel = [](double r2, double b2) { return b2 > 0 ? std::sqrt(r2 / b2) : 0.0; };
      st->defect_rel_residual[0] = rel(dn[0], dn[1]);
      st->defect_rel_residual[1] = rel(dn[2 * K], dn[2 * K + 1]);
    }
  } else {
    launch_u_stats(s->U, s->stream);
    if ((rc = s->cuda(cudaMemcpyAsync(red, s->U.red, sizeof(red), cudaMemcpyDeviceToHost, s->stream), "stats"))) return rc;
    if ((rc = s->sync("stats"))) return rc;
    st->mass = red[1];
    st->leaf_cells[0] = s->U.nc;
    st->active_cells = s->U.nc;
  }
  // the statistics are filled either way; the status reports a non-finite value
  if (nan_seen) return s->fail(DCG_E_NAN, device_error_text(st->device_error));
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
  if (which == 4 && s->ls_grid <= 0) return s->fail(DCG_E_INVALID, "no cooperative level solve on this device");
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
      case 4:
        if (s->ls_epoch == 3) s->solve_staged(level, 0, s->P.jacobi_iters);
        else launch_level_solve(s->D, level, 0, s->P.jacobi_iters, s->ls_grid, s->ls_epoch, s->stream);
        break;
      default: launch_divergence(s->D, s->stream); break;
    }
  };
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

int dcg_check_div6(uint64_t *mismatches, uint32_t *first) {
  if (!mismatches || !first) return DCG_E_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return DCG_E_CUDA;
  unsigned long long *d = nullptr, h[2] = {0, 0xFFFFFFFFull};
  if (cudaMalloc(&d, sizeof h) != cudaSuccess) return DCG_E_CUDA;
  cudaError_t e = cudaMemcpy(d, h, sizeof h, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    launch_check_div6(d, sms, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return DCG_E_CUDA;
  *mismatches = h[0];
  *first = (uint32_t)h[1];
  return DCG_OK;
}

int dcg_check_barrier_timeout(dcg_sim *s, uint32_t poll_limit) {
  if (bad(s) || s->mode != DCG_MODE_ADAPTIVE || poll_limit == 0 || poll_limit > (1u << 20)) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  const size_t bar_bytes = 4 * (64 + 32 * 18);
  int rc;
  if ((rc = s->cuda(cudaMemsetAsync(s->D.bar, 0, bar_bytes, s->stream), "barrier check"))) return rc;
  if ((rc = s->cuda((cudaError_t)launch_barrier_probe(s->D.bar, s->D.err, poll_limit, 2, s->stream),
                    "barrier check launch")))
    return rc;
  // the waiting CTA's arrival stays counted: clear the words for the next solve
  return s->cuda(cudaMemsetAsync(s->D.bar, 0, bar_bytes, s->stream), "barrier check");
}

size_t dcg_sizeof_params(void) { return sizeof(dcg_params); }
size_t dcg_sizeof_info(void) { return sizeof(dcg_info); }
size_t dcg_sizeof_stats(void) { return sizeof(dcg_stats); }

// ---- headless renderer -------------------------------------------------------
void dcg_default_render_params(dcg_render_params *rp, int32_t width, int32_t height) {
  std::memset(rp, 0, sizeof(*rp));
  rp->width = width;
  rp->height = height;
  rp->eye_dir[2] = 1.f;  // along +z
  rp->fov = 1.f;
  const float sx = .5f, sy = 1.f, sz = .3f, sn = std::sqrt(sx * sx + sy * sy + sz * sz);
  rp->sun_dir[0] = sx / sn; rp->sun_dir[1] = sy / sn; rp->sun_dir[2] = sz / sn;
  rp->aa_samples = 1;              // src/data/sim_params.cpp:24
  rp->channel = DCG_RENDER_FLUID;  // the displayed frame's channel, simulation.cpp:153
  rp->shadows = 1;                 // cpp:21
  rp->solids = 1;                  // cpp:20
  rp->precise = 1;                 // cpp:22
  rp->ambient = .3f;               // cpp:27
  for (int i = 0; i < 3; i++) rp->smoke_color[i] = .9f;  // cpp:30
  const float scene[3] = {107.f, 163.f, 204.f}, floor_[3] = {178.f, 158.f, 135.f};  // cpp:29,31
  for (int i = 0; i < 3; i++) {
    rp->scene_color[i] = scene[i] / 255.f;
    rp->floor_color[i] = floor_[i] / 255.f;
  }
}
int dcg_render(dcg_sim *s, const dcg_render_params *rp, float *rgba, int32_t where) {
  if (bad(s) || !rp || !rgba || rp->width <= 0 || rp->height <= 0 || rp->aa_samples < 1 || rp->channel < 0 ||
      rp->channel > DCG_RENDER_RESOLUTION)
    return DCG_E_INVALID;
  if (s->mode == DCG_MODE_UNIFORM && s->P.precision != DCG_PRECISION_FP32) return DCG_E_INVALID;
  RenderP R{};
  R.width = rp->width; R.height = rp->height; R.aa = rp->aa_samples; R.channel = rp->channel;
  R.shadows = rp->shadows; R.solids = rp->solids; R.precise = rp->precise;
  for (int i = 0; i < 3; i++) {
    R.eye[i] = rp->eye[i]; R.eye_dir[i] = rp->eye_dir[i]; R.sun[i] = rp->sun_dir[i];
    R.smoke[i] = rp->smoke_color[i]; R.scene[i] = rp->scene_color[i]; R.floor_[i] = rp->floor_color[i];
  }
  R.fov = rp->fov;
  R.ambient = rp->ambient;
  const size_t n = (size_t)rp->width * rp->height;
  float4 *out = reinterpret_cast<float4 *>(rgba);
  int rc;
  if (where != DCG_DEVICE) {
    if (s->render_cap < n) {
      if (s->render_tmp) cudaFree(s->render_tmp);
      s->render_tmp = nullptr;
      s->render_cap = 0;
      if ((rc = s->cuda(cudaMalloc(&s->render_tmp, n * 16), "render"))) return rc;
      s->render_cap = n;
    }
    out = reinterpret_cast<float4 *>(s->render_tmp);
  }
  if (s->mode == DCG_MODE_ADAPTIVE) launch_render_adaptive(s->D, R, out, s->stream);
  else launch_render_uniform(s->U, R, out, s->stream);
  if ((rc = s->check_launch("render"))) return rc;
  if (where != DCG_DEVICE &&
      (rc = s->cuda(cudaMemcpyAsync(rgba, out, n * 16, cudaMemcpyDeviceToHost, s->stream), "render")))
    return rc;
  return s->sync("render");
}
size_t dcg_sizeof_render_params(void) { return sizeof(dcg_render_params); }

// ---- memory-budget calculator -----------------------------------------------
int dcg_plan_bytes(const dcg_params *params, int32_t mode, int64_t *bytes) {
  if (!params || !bytes || (mode != DCG_MODE_ADAPTIVE && mode != DCG_MODE_UNIFORM)) return DCG_E_INVALID;
  dcg_sim s;
  s.P = *params;
  s.mode = mode;
  s.plan_only = true;
  const int rc = mode == DCG_MODE_ADAPTIVE ? s.create_adaptive() : s.create_uniform();
  if (rc) return rc;
  *bytes = (int64_t)s.bytes;
  return DCG_OK;
}
int dcg_blocks_for_budget(const dcg_params *params, int64_t budget_bytes, int64_t *max_blocks) {
  if (!params || !max_blocks || budget_bytes <= 0) return DCG_E_INVALID;
  dcg_params p = *params;
  auto fits = [&](int64_t b, int *rc) {
    p.max_blocks = b;
    int64_t n = 0;
    *rc = dcg_plan_bytes(&p, DCG_MODE_ADAPTIVE, &n);
    return *rc == DCG_OK && n <= budget_bytes;
  };
  // the smallest valid budget fills the coarsest level; budgets beyond the
  // full block count of every level leave blocks no level can use
  dcg_params q = *params;
  q.max_blocks = (1ll << 28) - 1;
  dcg_sim probe;
  probe.P = q;
  probe.plan_only = true;
  int rc = probe.create_adaptive();
  if (rc) return rc;
  long long lo = probe.D.g.full[probe.D.g.levels - 1], hi = 0;
  for (int l = 0; l < probe.D.g.levels; l++) hi += probe.D.g.full[l];
  // smallest budget the level split accepts (every level gets a block)
  for (long long a = lo, b = hi; ; ) {
    if (a >= b) {
      lo = a;
      break;
    }
    const long long mid = a + (b - a) / 2;
    int64_t n = 0;
    p.max_blocks = mid;
    if (dcg_plan_bytes(&p, DCG_MODE_ADAPTIVE, &n) == DCG_OK) b = mid;
    else a = mid + 1;
  }
  if (!fits(lo, &rc)) return rc ? rc : DCG_E_BUDGET;
  if (fits(hi, &rc)) {
    *max_blocks = hi;
    return DCG_OK;
  }
  while (hi - lo > 1) {
    const long long mid = lo + (hi - lo) / 2;
    if (fits(mid, &rc)) lo = mid;
    else hi = mid;
  }
  *max_blocks = lo;
  return DCG_OK;
}

// ---- state I/O -------------------------------------------------------------
namespace {
struct StateHeader {
  char magic[8];
  int32_t version, gx, gy, gz, levels, n_scalars, precision, pad;
  int64_t max_blocks, bytes, reserved;
};
static_assert(sizeof(StateHeader) == 64, "state header is 64 bytes");
const char kStateMagic[8] = {'D', 'C', 'G', 'S', 'T', 'A', 'T', 'E'};
}  // namespace

int dcg_state_bytes(dcg_sim *s, int64_t *bytes) {
  if (bad(s) || !bytes || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  size_t n = sizeof(StateHeader);
  for (auto &sec : s->state_sections()) n += sec.second;
  *bytes = (int64_t)n;
  return DCG_OK;
}
int dcg_save_state(dcg_sim *s, void *dst, int32_t where) {
  if (bad(s) || !dst || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  int64_t total = 0;
  dcg_state_bytes(s, &total);
  StateHeader h{};
  std::memcpy(h.magic, kStateMagic, 8);
  h.version = 1;
  h.gx = s->P.gx; h.gy = s->P.gy; h.gz = s->P.gz;
  h.levels = s->D.g.levels;
  h.n_scalars = s->P.n_scalars;
  h.precision = s->P.precision;
  h.max_blocks = s->D.g.B;
  h.bytes = total;
  const cudaMemcpyKind kind = where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  char *out = static_cast<char *>(dst);
  int rc;
  if (where == DCG_DEVICE) {
    if ((rc = s->cuda(cudaMemcpyAsync(out, &h, sizeof h, cudaMemcpyHostToDevice, s->stream), "save_state")))
      return rc;
  } else {
    std::memcpy(out, &h, sizeof h);
  }
  size_t off = sizeof h;
  for (auto &sec : s->state_sections()) {
    if ((rc = s->cuda(cudaMemcpyAsync(out + off, sec.first, sec.second, kind, s->stream), "save_state"))) return rc;
    off += sec.second;
  }
  return s->sync("save_state");
}
int dcg_load_state(dcg_sim *s, const void *src, int32_t where) {
  if (bad(s) || !src || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  StateHeader h{};
  const char *in = static_cast<const char *>(src);
  int rc;
  if (where == DCG_DEVICE) {
    if ((rc = s->cuda(cudaMemcpy(&h, in, sizeof h, cudaMemcpyDeviceToHost), "load_state"))) return rc;
  } else {
    std::memcpy(&h, in, sizeof h);
  }
  int64_t total = 0;
  dcg_state_bytes(s, &total);
  if (std::memcmp(h.magic, kStateMagic, 8) != 0 || h.version != 1 || h.gx != s->P.gx || h.gy != s->P.gy ||
      h.gz != s->P.gz || h.levels != s->D.g.levels || h.n_scalars != s->P.n_scalars ||
      h.precision != s->P.precision || h.max_blocks != s->D.g.B || h.bytes != total)
    return s->fail(DCG_E_INVALID, "state does not match this simulation's geometry, budget or formats");
  const cudaMemcpyKind kind = where == DCG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  size_t off = sizeof h;
  for (auto &sec : s->state_sections()) {
    if ((rc = s->cuda(cudaMemcpyAsync(sec.first, in + off, sec.second, kind, s->stream), "load_state"))) return rc;
    off += sec.second;
  }
  cudaMemsetAsync(s->D.ctr, 0, sizeof(long long) * C_COUNT, s->stream);
  cudaMemsetAsync(s->D.err, 0, 4, s->stream);
  return s->sync("load_state");
}

// ---- adjoint of the density path ------------------------------------------
int dcg_adjoint_step(dcg_sim *s, const float *lam_in, float *lam_out, float *lam_emission) {
  if (bad(s) || !lam_in || !lam_out || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  if (s->D.g.mixed) return s->fail(DCG_E_INVALID, "the adjoint is implemented for FP32 scalar storage");
  const size_t nc = (size_t)s->D.g.B * BV;
  int rc;
  if (!s->adj_tmp && (rc = s->alloc(&s->adj_tmp, nc))) return rc;
  if ((rc = s->cuda(cudaMemcpyAsync(s->adj_tmp, lam_in, nc * 4, cudaMemcpyDeviceToDevice, s->stream), "adjoint")))
    return rc;
  launch_adjoint_step(s->D, s->adj_tmp, lam_out, s->P.emission_n > 0 ? lam_emission : nullptr, s->sms, s->stream);
  return s->check_launch("adjoint_step");
}
// Full adjoint of one step: the handle holds the state before the step; the
// call records it, runs the step (stage by stage, the same kernels as
// dcg_step) and applies the transposes of its stages in reverse order.
int dcg_adjoint_step_full(dcg_sim *s, const float *lam_in, float *lam_out, float *lam_emission) {
  if (bad(s) || !lam_in || !lam_out || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  if (member_refused(s)) return DCG_E_INVALID;
  if (s->D.g.mixed) return s->fail(DCG_E_INVALID, "the adjoint is implemented for FP32 scalar storage");
  if (s->P.defect_passes) return s->fail(DCG_E_INVALID, "the full adjoint does not transpose the defect correction");
  const size_t B = (size_t)s->D.g.B, nc = B * BV;
  const int nq = s->P.n_scalars;
  int rc;
  if (!s->afull) {
    if ((rc = s->alloc(&s->afull, 19 * nc)) || (rc = s->alloc(&s->afull_pos, B)) ||
        (rc = s->alloc(&s->afull_parent, B)) || (rc = s->alloc(&s->afull_child, 8 * B)) ||
        (rc = s->alloc(&s->afull_nbr, 27 * B)))
      return rc;
  }
  float *V0 = s->afull, *Q0 = V0 + 3 * nc, *Q0P = Q0 + 3 * nc, *W0 = Q0P + 3 * nc, *LV = W0 + nc,
        *LQ = LV + 3 * nc, *LP = LQ + 3 * nc;
  auto cp = [&](void *dst, const void *src, size_t bytes) {
    if (!rc) rc = s->cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s->stream), "adjoint_step_full");
  };
  rc = 0;
  // the state before the step and the incoming adjoint
  for (int d = 0; d < 3; d++) cp(V0 + d * nc, s->D.v[d], nc * 4);
  for (int k = 0; k < nq; k++) cp(Q0 + k * nc, s->D.q[k], nc * 4);
  cp(W0, s->D.w, nc * 4);
  cp(s->afull_pos, s->D.pos, B * sizeof(int4));
  cp(s->afull_parent, s->D.parent, B * 4);
  cp(s->afull_child, s->D.child, 8 * B * 4);
  cp(s->afull_nbr, s->D.nbr, 27 * B * 4);
  cp(LV, lam_in, 3 * nc * 4);
  cp(LQ, lam_in + 3 * nc, nq * nc * 4);
  if (rc) return rc;
  Dev D0 = s->D;
  D0.pos = s->afull_pos;
  D0.parent = s->afull_parent;
  D0.child = s->afull_child;
  D0.nbr = s->afull_nbr;
  D0.w = W0;
  for (int d = 0; d < 3; d++) D0.v[d] = V0 + d * nc;
  for (int k = 0; k < nq; k++) D0.q[k] = Q0 + k * nc;
  // the step, keeping the scalars its advection reads (after the propagation)
  s->stage_advect_velocity();
  s->stage_adapt();
  for (int k = 0; k < nq; k++) cp(Q0P + k * nc, s->D.q[k], nc * 4);
  if (rc) return rc;
  s->stage_project(false);
  s->stage_advect_scalars();
  s->steps++;
  Dev DA = s->D;
  for (int k = 0; k < nq; k++) DA.q[k] = Q0P + k * nc;
  AdjFull A{LV, LQ, LP, LP + nc, LP + 2 * nc, lam_out, lam_out + 3 * nc};
  launch_adjoint_full_phase_a(DA, A, s->P.emission_n > 0 ? lam_emission : nullptr, s->P.jacobi_iters, s->sms,
                              s->stream);
  launch_adjoint_full_phase_b(D0, A, s->stream);
  return s->check_launch("adjoint_step_full");
}
int dcg_adjoint_dense(dcg_sim *s, const float *lam_dense, float *lam_cells) {
  if (bad(s) || !lam_dense || !lam_cells || s->mode != DCG_MODE_ADAPTIVE) return DCG_E_INVALID;
  launch_adjoint_dense(s->D, lam_dense, lam_cells, s->stream);
  return s->check_launch("adjoint_dense");
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Dense read-out without device allocation.
//
// dcg_get_dense stages the resampled volume in a device buffer that it
// cudaMallocs on its first call. Some callers cannot allocate at that point:
// hosts that hand the library a fixed device-memory budget up front and
// account for every byte it may take, and real-time loops that must not hit
// cudaMalloc's implicit device synchronisation in the middle of a frame.
// dcg_get_dense_noalloc runs the same resampling kernel but stages through the
// fixed array below, so the call itself allocates nothing. Like dcg_get_dense
// it waits for the handle's stream before it returns.
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
