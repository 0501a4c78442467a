// The reference's frame order (src/simulation.cpp:104-112: advectVelocity,
// adaptTopology, project, advectDensity) driven through the FluidSimulation
// adapter must give the same state as dcg_step on a handle made with
// dcg_default_params, bit for bit; and the adapter's render() into a CUDA
// surface must hold dcg_render's image. Exit status 0 on success.
#include <cstdio>
#include <cstring>
#include <vector>

#include "fluid_simulation_gb300.h"

static SimParams reference_defaults(int gx) {
  // SimParams::defaultParams (src/data/sim_params.cpp:4-34) for a gx-wide domain
  SimParams p;
  std::memset(&p, 0, sizeof p);
  p.dt = 3.f;
  p.dx = 10000.f / (float)gx;
  p.velocity_emission_rate = 150.f;
  p.density_emission_rate = 0.002f;
  p.emission_radius = 750.f;
  p.enable_additional_solids = false;
  p.render_solids = true;
  p.render_shadows = true;
  p.render_precise = true;
  p.render_channel = RenderChannel::Fluid;
  p.aa_samples = 1.f;
  p.ambient = .3f;
  p.floor_color = make_float3(178.f / 255.f, 158.f / 255.f, 135.f / 255.f);
  p.smoke_color = make_float3(.9f, .9f, .9f);
  p.scene_color = make_float3(107.f / 255.f, 163.f / 255.f, 204.f / 255.f);
  return p;
}

static int fail(const char *what) {
  std::fprintf(stderr, "FAIL: %s\n", what);
  return 1;
}

int main() {
  const int3 size = make_int3(32, 64, 32);
  const size_t blocks = 600;
  const int frames = 4;
  SimParams sp = reference_defaults(size.x);
  FluidSimulationGB300 sim(size, blocks, sp);
  sim.init();
  for (int f = 0; f < frames; f++) {
    sim.advectVelocity();
    sim.adaptTopology();
    sim.project();
    sim.advectDensity();
  }
  dcg_params p;
  dcg_default_params(&p, size.x, size.y, size.z, (int64_t)blocks);
  dcg_sim *ref = nullptr;
  if (dcg_create(&p, DCG_MODE_ADAPTIVE, &ref) != DCG_OK) return fail("dcg_create");
  if (dcg_step(ref, frames) != DCG_OK || dcg_sync(ref) != DCG_OK || dcg_sync(sim.handle()) != DCG_OK)
    return fail("dcg_step");
  dcg_info info;
  dcg_get_info(ref, &info);
  std::vector<float> a((size_t)info.num_cells), b((size_t)info.num_cells);
  const int fields[] = {DCG_FIELD_DENSITY, DCG_FIELD_VEL_X, DCG_FIELD_VEL_Y, DCG_FIELD_VEL_Z,
                        DCG_FIELD_FLUIDITY, DCG_FIELD_PRESSURE, DCG_FIELD_DIVERGENCE};
  for (int f : fields) {
    if (dcg_get_field(sim.handle(), f, a.data(), DCG_HOST) != DCG_OK ||
        dcg_get_field(ref, f, b.data(), DCG_HOST) != DCG_OK)
      return fail("dcg_get_field");
    if (std::memcmp(a.data(), b.data(), a.size() * sizeof(float)) != 0) {
      std::fprintf(stderr, "field %d differs\n", f);
      return fail("frame order through the adapter differs from dcg_step");
    }
  }
  // render into a CUDA surface of float4 texels (no graphics API involved)
  const int w = 64, h = 48;
  cudaChannelFormatDesc cd = cudaCreateChannelDesc<float4>();
  cudaArray_t arr = nullptr;
  if (cudaMallocArray(&arr, &cd, w, h, cudaArraySurfaceLoadStore) != cudaSuccess) return fail("cudaMallocArray");
  cudaResourceDesc rd;
  std::memset(&rd, 0, sizeof rd);
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = arr;
  cudaSurfaceObject_t surf = 0;
  if (cudaCreateSurfaceObject(&surf, &rd) != cudaSuccess) return fail("cudaCreateSurfaceObject");
  const float3 eye = make_float3(0.5f * size.x * sp.dx, 0.5f * size.y * sp.dx, -1.2f * size.z * sp.dx);
  const float3 dir = make_float3(0.f, 0.f, 1.f), sun = make_float3(0.4f, 0.8f, 0.45f);
  const float fov = 1.f;
  sim.render(surf, make_int2(w, h), eye, dir, fov, sun);
  std::vector<float> img((size_t)w * h * 4), want((size_t)w * h * 4);
  if (cudaMemcpy2DFromArray(img.data(), w * sizeof(float4), arr, 0, 0, w * sizeof(float4), h,
                            cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail("read the surface");
  dcg_render_params rp;
  dcg_default_render_params(&rp, w, h);
  rp.eye[0] = eye.x; rp.eye[1] = eye.y; rp.eye[2] = eye.z;
  rp.eye_dir[0] = dir.x; rp.eye_dir[1] = dir.y; rp.eye_dir[2] = dir.z;
  rp.sun_dir[0] = sun.x; rp.sun_dir[1] = sun.y; rp.sun_dir[2] = sun.z;
  rp.fov = fov;
  rp.channel = DCG_RENDER_FLUID;
  if (dcg_render(ref, &rp, want.data(), DCG_HOST) != DCG_OK) return fail("dcg_render");
  if (std::memcmp(img.data(), want.data(), img.size() * sizeof(float)) != 0)
    return fail("render() through the adapter differs from dcg_render");
  double sum = 0;
  for (float x : img) sum += x;
  if (!(sum > 0)) return fail("empty image");
  cudaDestroySurfaceObject(surf);
  cudaFreeArray(arr);
  dcg_destroy(ref);
  std::printf("adapter ok: %d frames bit-identical to dcg_step, render identical\n", frames);
  return 0;
}
