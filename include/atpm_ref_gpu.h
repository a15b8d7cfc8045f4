/*
 * atpm_ref_gpu.h -- the reference Thermal driver's GPU-module interface,
 * exported by binarytpm_gb300/driver/atpm_ref_gpu_shim.cpp over libatpm.
 *
 * The reference driver (3905/Thermal/NominalPole/main.cpp) declares these 27
 * functions itself (main.cpp:1850-2411) and links the module that defines
 * them (GPU_code.cu:600-1026).  Like that module, this interface is sized at
 * compile time: define REF_ASTNUMFACE, REF_NTAU and REF_NX to the driver's
 * ASTNUMFACE, NTAU and NX before including it (the crater has 61 vertices
 * and 100 sub-facets).  Linking the shim instead of GPU_code.cu is the whole
 * change: the driver's source is not touched.
 */
#ifndef ATPM_REF_GPU_H
#define ATPM_REF_GPU_H

#if !defined(REF_ASTNUMFACE) || !defined(REF_NTAU) || !defined(REF_NX)
#error "define REF_ASTNUMFACE, REF_NTAU and REF_NX (the driver's compile-time sizes)"
#endif

namespace atpm_ref {
const int SFCNUMVTX = 61;
const int SFCNUMFACE = 100;
/* GPU_code.cu:37-134 */
struct GPU_SfcVertex { float pos[3]; };
struct GPU_SfcFacet {
    int sfcvertices[3];
    float midpos[3];
    float trivector[2][3];
    float normcalc[3][3];
    float normal[3];
};
struct GPU_Surface { int NV, NF; GPU_SfcVertex* SV; GPU_SfcFacet* SF; };
struct Facet_Properties { bool sfc_converged; float albedo; float thermal_inertia; };
struct Roughness_Shadow {
    int shadow[REF_NTAU];
    float sfc_shadow[REF_NTAU][SFCNUMFACE];
    float sfc_illumvector[REF_NTAU][3];
    float sfc_illumangle[REF_NTAU][SFCNUMFACE];
};
struct Roughness_Illumination { float sfc_illumination[REF_NTAU][SFCNUMFACE]; };
struct Roughness_Globalillumination { float sfc_globalillumination[REF_NTAU][SFCNUMFACE]; };
struct Roughness_Globalheating { float sfc_globalheating[REF_NTAU][SFCNUMFACE]; };
struct Roughness_Temperatures {
    float sfc_stemp0[REF_NTAU][SFCNUMFACE];
    float sfc_stemp1[REF_NTAU][SFCNUMFACE];
    float sfc_temp[REF_NX + 1][SFCNUMFACE];
};
}  // namespace atpm_ref

extern "C" {
void set_cuda_device();                                             /* GPU_code.cu:600-605 */
void initialise_GPU_constants(float rot_period, float vf[atpm_ref::SFCNUMFACE][atpm_ref::SFCNUMFACE],
                              atpm_ref::GPU_Surface S);              /* 611-690 */
void initialise_GPU_facet_properties_arrays();                      /* 696-703 */
void initialise_GPU_shadow_arrays();                                /* 709-716 */
void initialise_GPU_illumination_arrays();                          /* 722-729 */
void initialise_GPU_globalillumination_arrays();                    /* 735-742 */
void initialise_GPU_globalheating_arrays();                         /* 748-755 */
void initialise_GPU_temperature_arrays();                           /* 761-768 */
void freeup_GPU_shadow_arrays();                                    /* 774-779 */
void freeup_GPU_globalillumination_arrays();                        /* 785-790 */
void freeup_GPU_globalheating_arrays();                             /* 796-801 */
void freeup_GPU_temperature_arrays();                               /* 807-812 */
void set_GPU_facet_properties(atpm_ref::Facet_Properties* FP_H);     /* 818-825 */
void load_GPU_globalillumination(atpm_ref::Roughness_Globalillumination* RGI_H);  /* 831-838 */
void load_GPU_globalheating(atpm_ref::Roughness_Globalheating* RGH_H);            /* 844-851 */
void obtain_GPU_facet_properties(atpm_ref::Facet_Properties* FP_H);  /* 857-863 */
void obtain_GPU_roughness_shadows(atpm_ref::Roughness_Shadow* RS_H); /* 869-876 */
void obtain_GPU_roughness_temperatures(atpm_ref::Roughness_Temperatures* RT_H);   /* 882-889 */
void obtain_GPU_roughness_illumination(atpm_ref::Roughness_Illumination* RI_H);   /* 895-903 */
void GPU_sfcpartialshadow(atpm_ref::Roughness_Shadow* RS_H);         /* 909-921 */
void GPU_single_scattering(float solar);                            /* 927-935 */
void GPU_multiple_scattering(float solar, float scattering_accuracy);  /* 941-949 */
void GPU_zero_temperatures();                                       /* 955-961 */
void GPU_initialise_temperatures(float EPS, float SIGMA);           /* 967-976 */
void GPU_inertia_difference(float EPS, float SIGMA, float TACC);    /* 982-998 */
void GPU_inst_equilibrium(float EPS, float SIGMA);                  /* 1004-1015 */
void GPU_converged(float TACC);                                     /* 1021-1026 */
}
#endif /* ATPM_REF_GPU_H */
