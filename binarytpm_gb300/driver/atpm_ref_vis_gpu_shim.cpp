// The reference Visibility driver's GPU module (3905/Visibility/NominalPole/
// GPU_code.cu:146-283: the crater partial-visibility kernel toward the
// observer) as a shim over libatpm's shadow-only crater.
//
// Compile it with the driver instead of GPU_code.cu, with the driver's sizes:
//   g++ -DREF_ASTNUMFACE=<ASTNUMFACE> -DREF_NTAU=<NTAU>
//       -I include main.cpp atpm_ref_vis_gpu_shim.cpp -L<dir of libatpm.so> -latpm
// The kernel is the Thermal module's sfcpartialshadow with the observer in
// place of the Sun, so the same device code serves both (REFERENCE precision:
// the module's float expressions without contraction).
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "atpm.h"
#include "atpm_ref_vis_gpu.h"

namespace {

using namespace atpm_ref_vis;
const int NF = REF_ASTNUMFACE, NTAU = REF_NTAU;

atpm_context* g_ctx = nullptr;
atpm_crater* g_cr = nullptr;

void check(atpm_status s, const char* what) {
    if (s != ATPM_OK) {
        std::fprintf(stderr, "atpm visibility module %s: %s (%s)\n", what, atpm_status_string(s), atpm_last_error());
        std::exit(2);
    }
}

atpm_crater* crater() {
    if (!g_ctx) check(atpm_context_create(0, &g_ctx), "context");
    if (!g_cr) check(atpm_crater_create(g_ctx, NF, NTAU, 0, SFCNUMFACE, ATPM_REFERENCE, &g_cr), "create");
    return g_cr;
}

template <class T>
void gather(const Roughness_Shadow* rs, size_t off, size_t per, std::vector<T>& out) {
    out.resize((size_t)NF * per);
    for (int f = 0; f < NF; ++f)
        std::memcpy(&out[(size_t)f * per], reinterpret_cast<const char*>(&rs[f]) + off, per * sizeof(T));
}
template <class T>
void scatter(Roughness_Shadow* rs, size_t off, size_t per, const std::vector<T>& in) {
    for (int f = 0; f < NF; ++f)
        std::memcpy(reinterpret_cast<char*>(&rs[f]) + off, &in[(size_t)f * per], per * sizeof(T));
}

}  // namespace

extern "C" {

void set_cuda_device() {
    if (!g_ctx) check(atpm_context_create(0, &g_ctx), "context");
}

void initialise_GPU_constants(GPU_Surface S) {
    std::vector<float> v((size_t)S.NV * 3), tri((size_t)SFCNUMFACE * 6);
    std::vector<int32_t> fac((size_t)SFCNUMFACE * 3);
    for (int i = 0; i < S.NV; ++i)
        for (int k = 0; k < 3; ++k) v[3 * i + k] = S.SV[i].pos[k];
    for (int j = 0; j < SFCNUMFACE; ++j)
        for (int k = 0; k < 3; ++k) {
            fac[3 * j + k] = S.SF[j].sfcvertices[k];
            tri[6 * j + k] = S.SF[j].trivector[0][k];
            tri[6 * j + 3 + k] = S.SF[j].trivector[1][k];
        }
    check(atpm_crater_set_model(crater(), S.NV, v.data(), fac.data(), tri.data(), nullptr, 0.0f), "constants");
}

void initialise_GPU_shadow_arrays() { crater(); }
void freeup_GPU_shadow_arrays() {}

void GPU_sfcpartialshadow(Roughness_Shadow* RS_H) {
    std::vector<int32_t> sh;
    std::vector<float> ssh, iv, ia;
    gather(RS_H, offsetof(Roughness_Shadow, shadow), (size_t)NTAU, sh);
    gather(RS_H, offsetof(Roughness_Shadow, sfc_shadow), (size_t)NTAU * SFCNUMFACE, ssh);
    gather(RS_H, offsetof(Roughness_Shadow, sfc_illumvector), (size_t)NTAU * 3, iv);
    gather(RS_H, offsetof(Roughness_Shadow, sfc_illumangle), (size_t)NTAU * SFCNUMFACE, ia);
    atpm_crater* c = crater();
    check(atpm_crater_set_array(c, 0, sh.data()), "shadow");
    check(atpm_crater_set_array(c, 1, ssh.data()), "shadow");
    check(atpm_crater_set_array(c, 2, iv.data()), "shadow");
    check(atpm_crater_set_array(c, 3, ia.data()), "shadow");
    check(atpm_crater_partial_shadow(c), "partial shadow");
}

void obtain_GPU_roughness_shadows(Roughness_Shadow* RS_H) {
    std::vector<int32_t> sh((size_t)NF * NTAU);
    std::vector<float> ssh((size_t)NF * NTAU * SFCNUMFACE), iv((size_t)NF * NTAU * 3), ia(ssh.size());
    atpm_crater* c = crater();
    check(atpm_crater_get_array(c, 0, sh.data()), "shadow");
    check(atpm_crater_get_array(c, 1, ssh.data()), "shadow");
    check(atpm_crater_get_array(c, 2, iv.data()), "shadow");
    check(atpm_crater_get_array(c, 3, ia.data()), "shadow");
    scatter(RS_H, offsetof(Roughness_Shadow, shadow), (size_t)NTAU, sh);
    scatter(RS_H, offsetof(Roughness_Shadow, sfc_shadow), (size_t)NTAU * SFCNUMFACE, ssh);
    scatter(RS_H, offsetof(Roughness_Shadow, sfc_illumvector), (size_t)NTAU * 3, iv);
    scatter(RS_H, offsetof(Roughness_Shadow, sfc_illumangle), (size_t)NTAU * SFCNUMFACE, ia);
}

}  // extern "C"
