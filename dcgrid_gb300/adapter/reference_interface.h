// reference_interface.h — the reference's simulation interface, restated for
// builds without the reference's source tree on the include path.
//
// fluid_simulation_gb300.h includes the reference's own headers
// (src/fluid_simulation.h, src/data/sim_params.h) when they are found;
// otherwise this file declares the same interface so the adapter and its
// tests build anywhere. The declarations must stay alike: the abstract class
// FluidSimulation (src/fluid_simulation.h:4-27: constructor from the grid
// size, init/reset/adaptTopology, the four stage methods, render into a CUDA
// surface, debugStats; protected size and numCells) and the SimParams fields
// the adapter reads (src/data/sim_params.h:4-47).
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

enum class RenderChannel { Fluid, Density, Velocity, Fluidity, Resolution };

struct SimParams {
  float dt;
  int gx, gy, gz;
  float dx, rdx;
  float velocity_emission_rate, density_emission_rate, emission_radius;
  bool enable_additional_solids;
  bool render_solids, render_shadows, render_precise;
  RenderChannel render_channel;
  float aa_samples;
  float ambient;
  float3 background_color, floor_color, smoke_color, scene_color;
};

class FluidSimulation {
 public:
  explicit FluidSimulation(const int3 &s) : size(s), numCells((size_t)s.x * s.y * s.z) {}
  virtual ~FluidSimulation() {}
  virtual void init() = 0;
  virtual void reset() = 0;
  virtual void adaptTopology() = 0;
  virtual void advectVelocity() = 0;
  virtual void project() = 0;
  virtual void projectLocal() = 0;
  virtual void advectDensity() = 0;
  virtual void render(cudaSurfaceObject_t dest, const int2 &resolution, const float3 &eyePos,
                      const float3 &eyeDir, const float &fov, const float3 &sunDir) = 0;
  virtual void debugStats() = 0;

 protected:
  int3 size;
  size_t numCells;
};
