// Link-time stand-ins for the extern "C" roughness GPU module of the
// reference's non-synchronous Thermal program (175706/Run-04/thermal_GPU.cu,
// declared at 175706/Run-04/thermal.cpp:2379-3459).  TEST INFRASTRUCTURE
// ONLY: the oracle builds that program with its roughness model switched off,
// so only set_cuda_device is reached; anything else stops the run loudly.
#include <cstdio>
#include <cstdlib>

namespace {
[[noreturn]] void unused(const char* f) {
    std::fprintf(stderr, "ref_nonsync_gpu_stub: %s called, but the roughness model is off in this build\n", f);
    std::abort();
}
}  // namespace

extern "C" {
void set_cuda_device() {}
void initialise_GPU_facet_properties_arrays() { unused("initialise_GPU_facet_properties_arrays"); }
void initialise_GPU_shadow_arrays() { unused("initialise_GPU_shadow_arrays"); }
void initialise_GPU_illumination_arrays() { unused("initialise_GPU_illumination_arrays"); }
void initialise_GPU_temperature_arrays() { unused("initialise_GPU_temperature_arrays"); }
void initialise_GPU_globalillumination_arrays() { unused("initialise_GPU_globalillumination_arrays"); }
void initialise_GPU_globalheating_arrays() { unused("initialise_GPU_globalheating_arrays"); }
void freeup_GPU_shadow_arrays() { unused("freeup_GPU_shadow_arrays"); }
void freeup_GPU_temperature_arrays() { unused("freeup_GPU_temperature_arrays"); }
void freeup_GPU_globalillumination_arrays() { unused("freeup_GPU_globalillumination_arrays"); }
void freeup_GPU_globalheating_arrays() { unused("freeup_GPU_globalheating_arrays"); }
void GPU_single_scattering(float) { unused("GPU_single_scattering"); }
void GPU_multiple_scattering(float, float) { unused("GPU_multiple_scattering"); }
void GPU_zero_temperatures() { unused("GPU_zero_temperatures"); }
void GPU_initialise_temperatures(float, float, float) { unused("GPU_initialise_temperatures"); }
void GPU_inertia_difference(float, float, float, float) { unused("GPU_inertia_difference"); }
void GPU_inst_equilibrium(float, float, float) { unused("GPU_inst_equilibrium"); }
void GPU_converged(float) { unused("GPU_converged"); }
void obtain_GPU_facet_properties(bool*, float*, float*, float*) { unused("obtain_GPU_facet_properties"); }
void set_GPU_facet_properties(bool*, float*, float*, float*) { unused("set_GPU_facet_properties"); }
void initialise_GPU_constants(float, void*, ...) { unused("initialise_GPU_constants"); }
void load_GPU_globalillumination(float*) { unused("load_GPU_globalillumination"); }
void load_GPU_globalheating(float*) { unused("load_GPU_globalheating"); }
void GPU_sfcpartialshadow(int*, float*, float*, float*) { unused("GPU_sfcpartialshadow"); }
void obtain_GPU_roughness_shadows(int*, float*, float*, float*) { unused("obtain_GPU_roughness_shadows"); }
void obtain_GPU_roughness_temperatures(float*, float*, float*) { unused("obtain_GPU_roughness_temperatures"); }
void obtain_GPU_roughness_illumination(float*) { unused("obtain_GPU_roughness_illumination"); }
}
