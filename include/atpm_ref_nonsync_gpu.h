/*
 * atpm_ref_nonsync_gpu.h -- the GPU-module interface of the reference's
 * non-synchronous binary Thermal program, exported by
 * binarytpm_gb300/driver/atpm_ref_nonsync_gpu_shim.cpp over libatpm.
 *
 * The program (175706/Run-04/thermal.cpp) declares these 27 functions itself
 * (thermal.cpp:2379-3459) and links the module that defines them
 * (175706/Run-04/thermal_GPU.cu:698-1279).  Unlike the synchronous module
 * (atpm_ref_gpu.h) every array crosses as a flat [facet][step][sub-facet]
 * float array, the facet properties carry a per-facet revolution count, and
 * the thermal calls take the IR absorptivity.  The module is sized at compile
 * time: define REF_ASTNUMFACE (the program's NUMROUGHFACE, the facets of one
 * part), REF_NTAU and REF_NX before including it (the crater has 61 vertices
 * and 100 sub-facets).
 */
#ifndef ATPM_REF_NONSYNC_GPU_H
#define ATPM_REF_NONSYNC_GPU_H

#if !defined(REF_ASTNUMFACE) || !defined(REF_NTAU) || !defined(REF_NX)
#error "define REF_ASTNUMFACE, REF_NTAU and REF_NX (the program's compile-time sizes)"
#endif

namespace atpm_ref_nonsync {
const int SFCNUMVTX = 61;
const int SFCNUMFACE = 100;
/* thermal.cpp:1065-1100 */
struct GPU_SfcVertex { float pos[3]; };
struct GPU_SfcFacet {
    int sfcvertices[3];
    float midpos[3];
    float trivector[2][3];
    float normcalc[3][3];
    float normal[3];
};
struct GPU_Surface { int NV, NF; GPU_SfcVertex* SV; GPU_SfcFacet* SF; };
}  // namespace atpm_ref_nonsync

extern "C" {
void set_cuda_device();                                             /* thermal_GPU.cu:698-702 */
void initialise_GPU_constants(float rot_period,
                              float vf[atpm_ref_nonsync::SFCNUMFACE][atpm_ref_nonsync::SFCNUMFACE],
                              atpm_ref_nonsync::GPU_Surface S);      /* 709-788 */
void initialise_GPU_facet_properties_arrays();                      /* 794-813 */
void initialise_GPU_shadow_arrays();                                /* 816-836 */
void initialise_GPU_illumination_arrays();                          /* 839-853 */
void initialise_GPU_globalillumination_arrays();                    /* 856-870 */
void initialise_GPU_globalheating_arrays();                         /* 873-887 */
void initialise_GPU_temperature_arrays();                           /* 890-907 */
void freeup_GPU_shadow_arrays();                                    /* 910-923 */
void freeup_GPU_globalillumination_arrays();                        /* 926-936 */
void freeup_GPU_globalheating_arrays();                             /* 939-949 */
void freeup_GPU_temperature_arrays();                               /* 952-966 */
/* [NF] each; numrevs = the facet's body's turns per model period */
void set_GPU_facet_properties(bool* sfc_converged, float* albedo, float* thermal_inertia,
                              float* numrevs);                      /* 969-990 */
void load_GPU_globalillumination(float* sfc_globalillumination);    /* 993-1009, [NF][NTAU][100] */
void load_GPU_globalheating(float* sfc_globalheating);              /* 1012-1028 */
void obtain_GPU_facet_properties(bool* sfc_converged, float* albedo, float* thermal_inertia,
                                 float* numrevs);                   /* 1031-1052 */
void obtain_GPU_roughness_shadows(int* shadow, float* sfc_shadow, float* sfc_illumvector,
                                  float* sfc_illumangle);           /* 1055-1077 */
void obtain_GPU_roughness_temperatures(float* sfc_stemp0, float* sfc_stemp1,
                                       float* sfc_temp);            /* 1080-1099, temp [NF][NX+1][100] */
/* returns the global illumination array, as the reference module does */
void obtain_GPU_roughness_illumination(float* sfc_globalillumination);  /* 1102-1118 */
void GPU_sfcpartialshadow(int* shadow, float* sfc_shadow, float* sfc_illumvector,
                          float* sfc_illumangle);                   /* 1121-1151 */
void GPU_single_scattering(float solar);                            /* 1154-1170 */
void GPU_multiple_scattering(float solar, float scattering_accuracy);  /* 1173-1189 */
void GPU_zero_temperatures();                                       /* 1192-1204 */
void GPU_initialise_temperatures(float EPS, float SIGMA, float IR_ABS);  /* 1207-1222 */
void GPU_inertia_difference(float EPS, float SIGMA, float IR_ABS, float TACC);  /* 1225-1246 */
void GPU_inst_equilibrium(float EPS, float SIGMA, float IR_ABS);    /* 1249-1266 */
void GPU_converged(float TACC);                                     /* 1269-1279 */
}
#endif /* ATPM_REF_NONSYNC_GPU_H */
