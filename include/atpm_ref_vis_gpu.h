/*
 * atpm_ref_vis_gpu.h -- the reference Visibility driver's GPU-module
 * interface (3905/Visibility/NominalPole/GPU_code.cu:146-283: crater partial
 * visibility toward the observer), exported by
 * binarytpm_gb300/driver/atpm_ref_vis_gpu_shim.cpp over libatpm's
 * shadow-only crater (atpm_crater_create with nx = 0).
 *
 * The driver (3905/Visibility/NominalPole/main.cpp:710-892) declares these six
 * functions itself; define REF_ASTNUMFACE and REF_NTAU to its ASTNUMFACE and
 * NTAU before including this header.  Linking the shim instead of
 * GPU_code.cu is the whole change.
 */
#ifndef ATPM_REF_VIS_GPU_H
#define ATPM_REF_VIS_GPU_H

#if !defined(REF_ASTNUMFACE) || !defined(REF_NTAU)
#error "define REF_ASTNUMFACE and REF_NTAU (the driver's compile-time sizes)"
#endif

namespace atpm_ref_vis {
const int SFCNUMVTX = 61;
const int SFCNUMFACE = 100;
/* GPU_code.cu:27-71 */
struct GPU_SfcVertex { float pos[3]; };
struct GPU_SfcFacet {
    int sfcvertices[3];
    float midpos[3];
    float trivector[2][3];
    float normcalc[3][3];
    float normal[3];
};
struct GPU_Surface { int NV, NF; GPU_SfcVertex* SV; GPU_SfcFacet* SF; };
struct Roughness_Shadow {
    int shadow[REF_NTAU];
    float sfc_shadow[REF_NTAU][SFCNUMFACE];
    float sfc_illumvector[REF_NTAU][3];
    float sfc_illumangle[REF_NTAU][SFCNUMFACE];
};
}  // namespace atpm_ref_vis

extern "C" {
void set_cuda_device();                                             /* GPU_code.cu:146-150 */
void initialise_GPU_constants(atpm_ref_vis::GPU_Surface S);          /* 157-228 */
void initialise_GPU_shadow_arrays();                                /* 234-241 */
void freeup_GPU_shadow_arrays();                                    /* 247-252 */
void obtain_GPU_roughness_shadows(atpm_ref_vis::Roughness_Shadow* RS_H);  /* 258-265 */
void GPU_sfcpartialshadow(atpm_ref_vis::Roughness_Shadow* RS_H);    /* 271-283 */
}
#endif /* ATPM_REF_VIS_GPU_H */
