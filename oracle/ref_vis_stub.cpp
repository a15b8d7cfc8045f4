// Link-time stand-ins for the six extern "C" symbols of the reference
// Visibility GPU module (3905/Visibility/NominalPole/GPU_code.cu:146-283).
// TEST INFRASTRUCTURE ONLY: the oracle builds the Visibility driver with its
// crater (roughness) visibility switched off, so only set_cuda_device may be
// reached; anything else stops the run loudly.
#include <cstdio>
#include <cstdlib>

namespace {
[[noreturn]] void unused(const char* f) {
    std::fprintf(stderr, "ref_vis_stub: %s called, but crater visibility is disabled in this build\n", f);
    std::abort();
}
struct GPU_Surface { int NV, NF; void* SV; void* SF; };
}  // namespace

extern "C" {
void set_cuda_device() {}
void initialise_GPU_constants(GPU_Surface) { unused("initialise_GPU_constants"); }
void initialise_GPU_shadow_arrays() { unused("initialise_GPU_shadow_arrays"); }
void freeup_GPU_shadow_arrays() { unused("freeup_GPU_shadow_arrays"); }
void obtain_GPU_roughness_shadows(void*) { unused("obtain_GPU_roughness_shadows"); }
void GPU_sfcpartialshadow(void*) { unused("GPU_sfcpartialshadow"); }
}
