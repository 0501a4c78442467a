// fluid_simulation_gb300.h — drop-in for the reference's FluidSimulationDCGrid
// (src/dcgrid/fluid_simulation_dcgrid.h:5-61) behind its abstract interface
// FluidSimulation (src/fluid_simulation.h:4-27), over the C ABI in dcg.h.
//
// A reference host replaces
//   m_simulation = new FluidSimulationDCGrid(size, m_maxNumBlocks);   (src/simulation.cpp:32-35)
// with
//   m_simulation = new FluidSimulationGB300(size, m_maxNumBlocks, m_params);
// and keeps its frame order (src/simulation.cpp:104-112) unchanged. The
// reference's constructor reads the global __constant__ SimParams; here the
// physics comes from the host's SimParams at construction and the render
// switches from it at every render(). Errors throw std::runtime_error with
// the library's message where the reference calls exit(1).
//
// Header-only; link with libdcgrid_gb300.so and the CUDA runtime. Include
// paths: the directory of dcg.h and, for the reference's own interface, the
// reference's src/ directory (else reference_interface.h restates it).
#pragma once
#if __has_include("fluid_simulation.h") && __has_include("data/sim_params.h")
#include "fluid_simulation.h"
#include "data/sim_params.h"
#else
#include "reference_interface.h"
#endif
#include <algorithm>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "dcg.h"

class FluidSimulationGB300 : public FluidSimulation {
 public:
  // sp is the host's live SimParams: physics is taken now, render switches at
  // every render()
  FluidSimulationGB300(const int3 &size, const size_t &maxNumBlocks, const SimParams &sp)
      : FluidSimulation(size), sp_(&sp) {
    dcg_params p;
    dcg_default_params(&p, size.x, size.y, size.z, (int64_t)maxNumBlocks);
    p.dt = sp.dt;
    p.dx = sp.dx;
    p.velocity_emission_rate = sp.velocity_emission_rate;
    p.density_emission_rate = sp.density_emission_rate;
    p.emission_radius = sp.emission_radius;
    p.solids = sp.enable_additional_solids ? DCG_SOLIDS_SPHERE : DCG_SOLIDS_NONE;
    const int rc = dcg_create(&p, DCG_MODE_ADAPTIVE, &sim_);
    if (rc != DCG_OK) throw std::runtime_error("dcg_create failed with status " + std::to_string(rc));
  }
  ~FluidSimulationGB300() override {
    dcg_destroy(sim_);
    if (rgba_) cudaFree(rgba_);
  }
  FluidSimulationGB300(const FluidSimulationGB300 &) = delete;
  FluidSimulationGB300 &operator=(const FluidSimulationGB300 &) = delete;

  // FluidSimulationDCGrid::init and ::reset (fluid_simulation_dcgrid.cu:190-261):
  // both leave the simulation as after construction
  void init() override { check(dcg_reset(sim_)); }
  void reset() override { check(dcg_reset(sim_)); }
  void adaptTopology() override { check(dcg_adapt(sim_)); }
  void advectVelocity() override { check(dcg_advect_velocity(sim_)); }
  void project() override { check(dcg_project(sim_)); }
  void projectLocal() override { check(dcg_project_local(sim_)); }
  void advectDensity() override { check(dcg_advect_scalars(sim_)); }

  // the reference ray-marches into a surface of float4 texels
  // (dcgrid_rendering.cu:91); here dcg_render fills a device image that is
  // copied into the surface's array
  void render(cudaSurfaceObject_t dest, const int2 &res, const float3 &eye, const float3 &dir, const float &fov,
              const float3 &sun) override {
    dcg_render_params rp;
    dcg_default_render_params(&rp, res.x, res.y);
    const float3 v[6] = {eye, dir, sun, sp_->smoke_color, sp_->scene_color, sp_->floor_color};
    float *o[6] = {rp.eye, rp.eye_dir, rp.sun_dir, rp.smoke_color, rp.scene_color, rp.floor_color};
    for (int k = 0; k < 6; k++) {
      o[k][0] = v[k].x;
      o[k][1] = v[k].y;
      o[k][2] = v[k].z;
    }
    rp.fov = fov;
    rp.channel = (int32_t)sp_->render_channel;  // the same order as DCG_RENDER_*
    rp.aa_samples = std::max(1, (int32_t)sp_->aa_samples);
    rp.shadows = sp_->render_shadows;
    rp.solids = sp_->render_solids;
    rp.precise = sp_->render_precise;
    rp.ambient = sp_->ambient;
    const size_t n = (size_t)res.x * res.y;
    if (rgba_n_ < n) {
      if (rgba_) cudaFree(rgba_);
      rgba_ = nullptr;
      rgba_n_ = 0;
      if (cudaMalloc(&rgba_, n * sizeof(float4)) != cudaSuccess) throw std::runtime_error("render image");
      rgba_n_ = n;
    }
    check(dcg_render(sim_, &rp, reinterpret_cast<float *>(rgba_), DCG_DEVICE));
    cudaResourceDesc rd;
    if (cudaGetSurfaceObjectResourceDesc(&rd, dest) != cudaSuccess || rd.resType != cudaResourceTypeArray ||
        cudaMemcpy2DToArray(rd.res.array.array, 0, 0, rgba_, res.x * sizeof(float4), res.x * sizeof(float4),
                            res.y, cudaMemcpyDeviceToDevice) != cudaSuccess)
      throw std::runtime_error("render: copy into the surface's array failed");
  }
  // FluidSimulationDCGrid::debugStats (fluid_simulation_dcgrid.cu:517-529)
  void debugStats() override {
    dcg_stats st;
    check(dcg_get_stats(sim_, &st));
    std::printf("Residual: %g\n", st.residual);
  }

  // the C handle, for calls the reference interface does not have (fields,
  // statistics, graphs)
  dcg_sim *handle() const { return sim_; }

 private:
  void check(int rc) {
    if (rc != DCG_OK) throw std::runtime_error(dcg_last_error_string(sim_));
  }
  const SimParams *sp_;
  dcg_sim *sim_ = nullptr;
  float4 *rgba_ = nullptr;
  size_t rgba_n_ = 0;
};
