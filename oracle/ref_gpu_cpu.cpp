// CPU restatement of the reference's Thermal GPU roughness module
// (3905/Thermal/NominalPole/GPU_code.cu).  TEST INFRASTRUCTURE ONLY: it lets
// the reference's own Thermal driver (compiled from a scratch copy by
// oracle/refbuild.py) link and run on a host without a GPU.  Every kernel is
// executed as a loop over blocks (facets) and threads (crater sub-facets),
// keeping the kernel's arithmetic order; nvcc contracts multiply-adds in the
// original, this restatement does not, so crater results agree with the GPU
// module to float rounding only.
//
// Sizes come from -DREF_ASTNUMFACE / -DREF_NTAU / -DREF_NX (the reference
// fixes them as compile-time constants, GPU_code.cu:6-12).
//
// With -DREF_VISIBILITY_MODULE the file instead provides the six symbols of
// the Visibility driver's GPU module (3905/Visibility/NominalPole/
// GPU_code.cu:146-283), whose partial-visibility kernel is the same
// sfcpartialshadow toward the observer.
//
// With -DREF_NONSYNC_MODULE it provides the 27 symbols of the non-synchronous
// binary program's module instead (175706/Run-04/thermal_GPU.cu:698-1279):
// the same kernels over flat [facet][step][sub-facet] arrays, with each
// facet's revolution count in the time step and skin factor
// (thermal_GPU.cu:448-450, 539) and the IR absorptivity on the sub-facets'
// mutual emission (thermal_GPU.cu:390, 521, 615).  The synchronous module is
// the case of one revolution and absorptivity 1, whose products are exact, so
// one set of kernels serves both.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>

#ifndef REF_ASTNUMFACE
#error "REF_ASTNUMFACE required"
#endif
#if defined(REF_VISIBILITY_MODULE) && !defined(REF_NX)
#define REF_NX 1
#endif

namespace {
const int ASTNUMFACE = REF_ASTNUMFACE;
const int SFCNUMVTX = 61;
const int SFCNUMFACE = 100;
const int NTAU = REF_NTAU;
const int NX = REF_NX;
const int m = 10;

// Layouts identical to GPU_code.cu:37-134 (the driver passes these structs).
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
    int shadow[NTAU];
    float sfc_shadow[NTAU][SFCNUMFACE];
    float sfc_illumvector[NTAU][3];
    float sfc_illumangle[NTAU][SFCNUMFACE];
};
struct Roughness_Illumination { float sfc_illumination[NTAU][SFCNUMFACE]; };
struct Roughness_Globalillumination { float sfc_globalillumination[NTAU][SFCNUMFACE]; };
struct Roughness_Globalheating { float sfc_globalheating[NTAU][SFCNUMFACE]; };
struct Roughness_Temperatures {
    float sfc_stemp0[NTAU][SFCNUMFACE];
    float sfc_stemp1[NTAU][SFCNUMFACE];
    float sfc_temp[NX + 1][SFCNUMFACE];
};

// "device" state (GPU_code.cu:14-31, 140-146)
float c_vertex[SFCNUMVTX][3];
int c_facet[SFCNUMFACE][3];
float c_trivector[SFCNUMFACE][2][3];
float c_mult[m * m][2];
float c_PI;
float c_rot_period;
float* vf_D = nullptr;
Facet_Properties* FP_D = nullptr;
float* NR_D = nullptr;      // per-facet revolution counts (non-synchronous module)
float c_ir_abs = 1.0f;      // IR absorptivity (non-synchronous module)
Roughness_Shadow* RS_D = nullptr;
Roughness_Illumination* RI_D = nullptr;
Roughness_Globalillumination* RGI_D = nullptr;
Roughness_Globalheating* RGH_D = nullptr;
Roughness_Temperatures* RT_D = nullptr;

template <class T> T* alloc(size_t n) {
    T* p = static_cast<T*>(std::calloc(n, sizeof(T)));
    if (!p) { std::fprintf(stderr, "ref_gpu_cpu: out of memory\n"); std::abort(); }
    return p;
}

// GPU_code.cu:152-210
void k_sfcpartialshadow(int b, int step) {
    Roughness_Shadow& R = RS_D[b];
    if (R.shadow[step] != 1) return;
    float sv[3] = {R.sfc_illumvector[step][0], R.sfc_illumvector[step][1], R.sfc_illumvector[step][2]};
    float s = sqrtf((sv[0] * sv[0]) + (sv[1] * sv[1]));
    sv[0] = sv[0] / s; sv[1] = sv[1] / s; sv[2] = sv[2] / s;
    const float crater_radius = 10.0f;
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float sh = R.sfc_shadow[step][t];
        float a = fabsf(sv[2]) / sqrtf((sv[0] * sv[0]) + (sv[1] * sv[1]));
        for (int p = 0; p != m * m; ++p) {
            float mp[3];
            for (int k = 0; k < 3; ++k)
                mp[k] = c_vertex[c_facet[t][2]][k] + (c_mult[p][0] * c_trivector[t][0][k]) +
                        (c_mult[p][1] * c_trivector[t][1][k]);
            float tc1 = (-1.0f * sv[1] * mp[0]) + (sv[0] * mp[1]);
            float rad = sqrtf((crater_radius * crater_radius) - (tc1 * tc1));
            float tc0 = (sv[0] * mp[0]) + (sv[1] * mp[1]) - rad;
            if (mp[2] <= (a * tc0) && sh != 0.0f) sh = sh - (1.0f / (float)(m * m));
            if (sh < 0.0f) sh = 0.0f;
        }
        R.sfc_shadow[step][t] = sh;
    }
}

// GPU_code.cu:216-246
void k_single_scattering(int b, float solar, int step) {
    float albedo = FP_D[b].albedo;
    float ill[SFCNUMFACE];
    for (int t = 0; t < SFCNUMFACE; ++t)
        ill[t] = (solar * RS_D[b].sfc_shadow[step][t] * RS_D[b].sfc_illumangle[step][t]) +
                 RGI_D[b].sfc_globalillumination[step][t];
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float tot = ill[t];
        for (int i = 0; i != SFCNUMFACE; ++i) tot = tot + (vf_D[(i * SFCNUMFACE) + t] * albedo * ill[i]);
        if (tot <= 0.0f) tot = 0.0f;
        RI_D[b].sfc_illumination[step][t] = tot;
    }
}

// GPU_code.cu:252-304 (Jacobi iteration, barrier-separated)
void k_multiple_scattering(int b, float solar, float acc, int step) {
    float albedo = FP_D[b].albedo;
    float solarpower[SFCNUMFACE], pold[SFCNUMFACE], pnew[SFCNUMFACE];
    for (int t = 0; t < SFCNUMFACE; ++t) {
        solarpower[t] = (solar * RS_D[b].sfc_illumangle[step][t] * RS_D[b].sfc_shadow[step][t]) +
                        RGI_D[b].sfc_globalillumination[step][t];
        pold[t] = albedo * RI_D[b].sfc_illumination[step][t];
    }
    for (int it = 0; it < 100000; ++it) {
        int test = 0;
        for (int t = 0; t < SFCNUMFACE; ++t) {
            float sum = 0.0f;
            for (int i = 0; i != SFCNUMFACE; ++i) sum = sum + (vf_D[(i * SFCNUMFACE) + t] * pold[i]);
            pnew[t] = albedo * (solarpower[t] + sum);
        }
        for (int t = 0; t < SFCNUMFACE; ++t) {
            if (fabsf(pnew[t] - pold[t]) > acc) test = test + 1;
            pold[t] = pnew[t];
        }
        if (test == 0) break;
    }
    for (int t = 0; t < SFCNUMFACE; ++t) RI_D[b].sfc_illumination[step][t] = pnew[t] / albedo;
}

// GPU_code.cu:328-371
void k_initialise_temperatures(int b, float ES) {
    const float IR = c_ir_abs;
    float albedo = FP_D[b].albedo;
    float st0[SFCNUMFACE];
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float temp = 0.0f;
        for (int s = 0; s != NTAU; ++s)
            temp = temp + ((1.0f / NTAU) * (((1.0f - albedo) * RI_D[b].sfc_illumination[s][t]) +
                                           RGH_D[b].sfc_globalheating[s][t]));
        st0[t] = powf(temp / (ES), 0.25f);
    }
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float sh = 0.0f;
        for (int i = 0; i != SFCNUMFACE; ++i) sh = sh + (IR * ES * powf(st0[i], 4.0f) * vf_D[(i * SFCNUMFACE) + t]);
        float temp = 0.0f;
        for (int s = 0; s != NTAU; ++s)
            temp = temp + ((1.0f / NTAU) * (((1.0f - albedo) * RI_D[b].sfc_illumination[s][t]) +
                                           RGH_D[b].sfc_globalheating[s][t] + sh));
        temp = powf(temp / (ES), 0.25f);
        for (int i = 0; i != NX + 1; ++i) RT_D[b].sfc_temp[i][t] = temp;
        for (int s = 0; s != NTAU; ++s) { RT_D[b].sfc_stemp0[s][t] = temp; RT_D[b].sfc_stemp1[s][t] = temp; }
    }
}

// facet b's turns per model period: 1 in the synchronous module
float revs(int b) { return NR_D ? NR_D[b] : 1.0f; }

// GPU_code.cu:377-412 (the out-of-range read of row NX+1 at line 403 is not
// reproduced); non-synchronous: thermal_GPU.cu:430-478
void k_finite_difference(int b) {
    if (FP_D[b].sfc_converged) return;
    float DZ = 8.0f / NX, DTAU = (2.0f * c_PI * revs(b)) / NTAU, M0 = DTAU / (DZ * DZ);
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float (*T)[SFCNUMFACE] = RT_D[b].sfc_temp;
        float t0 = T[0][t], t1 = T[1][t], t2 = T[2][t];
        for (int i = 1; i != NX; ++i) {
            T[i][t] = t1 + (M0 * (t2 - (2.0f * t1) + t0));
            t0 = t1; t1 = t2;
            if (i + 2 <= NX) t2 = T[i + 2][t];
        }
        T[NX][t] = T[NX - 1][t];
    }
}

// GPU_code.cu:418-490; non-synchronous: thermal_GPU.cu:485-574
void k_boundary_condition(int b, float ES, float TACC, int step) {
    if (FP_D[b].sfc_converged) return;
    const float IR = c_ir_abs;
    float albedo = FP_D[b].albedo, ti = FP_D[b].thermal_inertia, nr = revs(b);
    float stemp[SFCNUMFACE];
    Roughness_Temperatures& R = RT_D[b];
    for (int t = 0; t < SFCNUMFACE; ++t) {
        stemp[t] = R.sfc_stemp1[step][t];
        R.sfc_stemp0[step][t] = stemp[t];
        stemp[t] = IR * ES * powf(stemp[t], 4.0f);
    }
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float TR0 = R.sfc_temp[0][t], TR1 = TR0, temp = R.sfc_temp[1][t];
        float ill = RI_D[b].sfc_illumination[step][t];
        float inc = RGH_D[b].sfc_globalheating[step][t];
        for (int i = 0; i != SFCNUMFACE; ++i) inc = inc + (stemp[i] * vf_D[(i * SFCNUMFACE) + t]);
        float DT = 1.0f, DZ = 8.0f / NX;
        float M1 = ti * sqrtf(2.0f * c_PI * nr / c_rot_period) / DZ;
        float M2 = ((1.0f - albedo) * ill) + inc;
        for (int it = 0; DT >= TACC && it < 1000; ++it) {
            float SBC = M2 + (M1 * (temp - TR0)) - (ES * TR0 * TR0 * TR0 * TR0);
            float SBCD = M1 + (4.0f * ES * TR0 * TR0 * TR0);
            TR1 = TR0 + (SBC / SBCD);
            DT = fabsf(TR1 - TR0);
            TR0 = TR1;
        }
        R.sfc_temp[0][t] = TR1;
        R.sfc_stemp1[step][t] = TR1;
    }
}

// GPU_code.cu:496-548; non-synchronous: thermal_GPU.cu:581-641
void k_inst_equilibrium(int b, float ES, int step) {
    if (FP_D[b].sfc_converged) return;
    const float IR = c_ir_abs;
    float albedo = FP_D[b].albedo;
    float stemp[SFCNUMFACE];
    Roughness_Temperatures& R = RT_D[b];
    for (int t = 0; t < SFCNUMFACE; ++t) {
        stemp[t] = R.sfc_stemp1[step][t];
        R.sfc_stemp0[step][t] = stemp[t];
        stemp[t] = IR * ES * powf(stemp[t], 4.0f);
    }
    for (int t = 0; t < SFCNUMFACE; ++t) {
        float inc = RGH_D[b].sfc_globalheating[step][t];
        for (int i = 0; i != SFCNUMFACE; ++i) inc = inc + (stemp[i] * vf_D[(i * SFCNUMFACE) + t]);
        float ill = RI_D[b].sfc_illumination[step][t];
        R.sfc_stemp1[step][t] = powf(((((1.0f - albedo) * ill) + inc) / (ES)), 0.25f);
    }
}

// GPU_code.cu:554-594
void k_converged(int b, float TACC) {
    if (FP_D[b].sfc_converged) return;
    bool conv = true;
    for (int t = 0; t < SFCNUMFACE; ++t)
        for (int s = 0; s != NTAU; ++s)
            if (fabsf(RT_D[b].sfc_stemp0[s][t] - RT_D[b].sfc_stemp1[s][t]) >= TACC) conv = false;
    FP_D[b].sfc_converged = conv;
}
}  // namespace

#ifdef REF_VISIBILITY_MODULE
namespace {
void set_constants(const GPU_Surface& S_H);
}
// ---- the six entry points of the Visibility module (GPU_code.cu:146-283) ----
extern "C" {
void set_cuda_device() {}
void initialise_GPU_constants(GPU_Surface S_H) { set_constants(S_H); }
void initialise_GPU_shadow_arrays() { RS_D = alloc<Roughness_Shadow>(ASTNUMFACE); }
void freeup_GPU_shadow_arrays() { std::free(RS_D); RS_D = nullptr; }
void obtain_GPU_roughness_shadows(Roughness_Shadow* H) { std::memcpy(H, RS_D, sizeof(*H) * ASTNUMFACE); }
void GPU_sfcpartialshadow(Roughness_Shadow* RS_H) {
    std::memcpy(RS_D, RS_H, sizeof(Roughness_Shadow) * ASTNUMFACE);
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_sfcpartialshadow(b, step);
    }
}
}
#elif defined(REF_NONSYNC_MODULE)
namespace {
void set_constants(const GPU_Surface& S_H);
void run_steps(void (*k)(int, float, int), float x) {
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k(b, x, step);
    }
}
}
// ---- the 27 entry points of the non-synchronous module
// (175706/Run-04/thermal_GPU.cu:698-1279): flat arrays in the layout of the
// synchronous module's per-facet structs, copied field by field ----
extern "C" {
void set_cuda_device() {}

void initialise_GPU_constants(float rot_period_H, float viewfactors_H[SFCNUMFACE][SFCNUMFACE], GPU_Surface S_H) {
    c_PI = 4.0f * atanf(1.0f);
    c_rot_period = rot_period_H;
    if (!vf_D) vf_D = alloc<float>(SFCNUMFACE * SFCNUMFACE);
    std::memcpy(vf_D, viewfactors_H, sizeof(float) * SFCNUMFACE * SFCNUMFACE);
    set_constants(S_H);
}
void initialise_GPU_facet_properties_arrays() {
    FP_D = alloc<Facet_Properties>(ASTNUMFACE);
    NR_D = alloc<float>(ASTNUMFACE);
}
void initialise_GPU_shadow_arrays() { RS_D = alloc<Roughness_Shadow>(ASTNUMFACE); }
void initialise_GPU_illumination_arrays() { RI_D = alloc<Roughness_Illumination>(ASTNUMFACE); }
void initialise_GPU_globalillumination_arrays() { RGI_D = alloc<Roughness_Globalillumination>(ASTNUMFACE); }
void initialise_GPU_globalheating_arrays() { RGH_D = alloc<Roughness_Globalheating>(ASTNUMFACE); }
void initialise_GPU_temperature_arrays() { RT_D = alloc<Roughness_Temperatures>(ASTNUMFACE); }
void freeup_GPU_shadow_arrays() { std::free(RS_D); RS_D = nullptr; }
void freeup_GPU_globalillumination_arrays() { std::free(RGI_D); RGI_D = nullptr; }
void freeup_GPU_globalheating_arrays() { std::free(RGH_D); RGH_D = nullptr; }
void freeup_GPU_temperature_arrays() { std::free(RT_D); RT_D = nullptr; }

void set_GPU_facet_properties(bool* conv, float* albedo, float* ti, float* numrevs) {
    for (int b = 0; b < ASTNUMFACE; ++b) {
        FP_D[b].sfc_converged = conv[b];
        FP_D[b].albedo = albedo[b];
        FP_D[b].thermal_inertia = ti[b];
        NR_D[b] = numrevs[b];
    }
}
void obtain_GPU_facet_properties(bool* conv, float* albedo, float* ti, float* numrevs) {
    for (int b = 0; b < ASTNUMFACE; ++b) {
        conv[b] = FP_D[b].sfc_converged;
        albedo[b] = FP_D[b].albedo;
        ti[b] = FP_D[b].thermal_inertia;
        numrevs[b] = NR_D[b];
    }
}
void load_GPU_globalillumination(float* H) { std::memcpy(RGI_D, H, sizeof(Roughness_Globalillumination) * ASTNUMFACE); }
void load_GPU_globalheating(float* H) { std::memcpy(RGH_D, H, sizeof(Roughness_Globalheating) * ASTNUMFACE); }

void GPU_sfcpartialshadow(int* shadow, float* sfc_shadow, float* sfc_illumvector, float* sfc_illumangle) {
    const size_t ns = (size_t)NTAU * SFCNUMFACE;
    for (int b = 0; b < ASTNUMFACE; ++b) {
        std::memcpy(RS_D[b].shadow, shadow + (size_t)b * NTAU, sizeof(int) * NTAU);
        std::memcpy(RS_D[b].sfc_shadow, sfc_shadow + b * ns, sizeof(float) * ns);
        std::memcpy(RS_D[b].sfc_illumvector, sfc_illumvector + (size_t)b * NTAU * 3, sizeof(float) * NTAU * 3);
        std::memcpy(RS_D[b].sfc_illumangle, sfc_illumangle + b * ns, sizeof(float) * ns);
    }
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_sfcpartialshadow(b, step);
    }
}
void obtain_GPU_roughness_shadows(int* shadow, float* sfc_shadow, float* sfc_illumvector, float* sfc_illumangle) {
    const size_t ns = (size_t)NTAU * SFCNUMFACE;
    for (int b = 0; b < ASTNUMFACE; ++b) {
        std::memcpy(shadow + (size_t)b * NTAU, RS_D[b].shadow, sizeof(int) * NTAU);
        std::memcpy(sfc_shadow + b * ns, RS_D[b].sfc_shadow, sizeof(float) * ns);
        std::memcpy(sfc_illumvector + (size_t)b * NTAU * 3, RS_D[b].sfc_illumvector, sizeof(float) * NTAU * 3);
        std::memcpy(sfc_illumangle + b * ns, RS_D[b].sfc_illumangle, sizeof(float) * ns);
    }
}
void obtain_GPU_roughness_temperatures(float* stemp0, float* stemp1, float* temp) {
    const size_t ns = (size_t)NTAU * SFCNUMFACE, nd = (size_t)(NX + 1) * SFCNUMFACE;
    for (int b = 0; b < ASTNUMFACE; ++b) {
        std::memcpy(stemp0 + b * ns, RT_D[b].sfc_stemp0, sizeof(float) * ns);
        std::memcpy(stemp1 + b * ns, RT_D[b].sfc_stemp1, sizeof(float) * ns);
        std::memcpy(temp + b * nd, RT_D[b].sfc_temp, sizeof(float) * nd);
    }
}
// thermal_GPU.cu:1102-1118 copies back the global-illumination array
void obtain_GPU_roughness_illumination(float* H) {
    std::memcpy(H, RGI_D, sizeof(Roughness_Globalillumination) * ASTNUMFACE);
}

void GPU_single_scattering(float solar) { run_steps(k_single_scattering, solar); }
void GPU_multiple_scattering(float solar, float acc) {
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_multiple_scattering(b, solar, acc, step);
    }
}
void GPU_zero_temperatures() {
    for (int b = 0; b < ASTNUMFACE; ++b) std::memset(&RT_D[b], 0, sizeof(Roughness_Temperatures));
}
void GPU_initialise_temperatures(float EPS, float SIGMA, float IR_ABS) {
    float ES = EPS * SIGMA;
    c_ir_abs = IR_ABS;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < ASTNUMFACE; ++b) k_initialise_temperatures(b, ES);
}
void GPU_inertia_difference(float EPS, float SIGMA, float IR_ABS, float TACC) {
    float ES = EPS * SIGMA, TACC2 = TACC / 10.0f;
    c_ir_abs = IR_ABS;
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) { k_finite_difference(b); k_boundary_condition(b, ES, TACC2, step); }
    }
}
void GPU_inst_equilibrium(float EPS, float SIGMA, float IR_ABS) {
    c_ir_abs = IR_ABS;
    run_steps(k_inst_equilibrium, EPS * SIGMA);
}
void GPU_converged(float TACC) {
#pragma omp parallel for schedule(static)
    for (int b = 0; b < ASTNUMFACE; ++b) k_converged(b, TACC);
}
}
#else
namespace {
void set_constants(const GPU_Surface& S_H);
}
// ---- the 27 extern "C" entry points (GPU_code.cu:600-1026) ----
extern "C" {
void set_cuda_device() {}

void initialise_GPU_constants(float rot_period_H, float viewfactors_H[SFCNUMFACE][SFCNUMFACE], GPU_Surface S_H) {
    c_PI = 4.0f * atanf(1.0f);
    c_rot_period = rot_period_H;
    if (!vf_D) vf_D = alloc<float>(SFCNUMFACE * SFCNUMFACE);
    std::memcpy(vf_D, viewfactors_H, sizeof(float) * SFCNUMFACE * SFCNUMFACE);
    set_constants(S_H);
}
void initialise_GPU_facet_properties_arrays() { FP_D = alloc<Facet_Properties>(ASTNUMFACE); }
void initialise_GPU_shadow_arrays() { RS_D = alloc<Roughness_Shadow>(ASTNUMFACE); }
void initialise_GPU_illumination_arrays() { RI_D = alloc<Roughness_Illumination>(ASTNUMFACE); }
void initialise_GPU_globalillumination_arrays() { RGI_D = alloc<Roughness_Globalillumination>(ASTNUMFACE); }
void initialise_GPU_globalheating_arrays() { RGH_D = alloc<Roughness_Globalheating>(ASTNUMFACE); }
void initialise_GPU_temperature_arrays() { RT_D = alloc<Roughness_Temperatures>(ASTNUMFACE); }
void freeup_GPU_shadow_arrays() { std::free(RS_D); RS_D = nullptr; }
void freeup_GPU_globalillumination_arrays() { std::free(RGI_D); RGI_D = nullptr; }
void freeup_GPU_globalheating_arrays() { std::free(RGH_D); RGH_D = nullptr; }
void freeup_GPU_temperature_arrays() { std::free(RT_D); RT_D = nullptr; }
void set_GPU_facet_properties(Facet_Properties* FP_H) { std::memcpy(FP_D, FP_H, sizeof(Facet_Properties) * ASTNUMFACE); }
void load_GPU_globalillumination(Roughness_Globalillumination* H) { std::memcpy(RGI_D, H, sizeof(*H) * ASTNUMFACE); }
void load_GPU_globalheating(Roughness_Globalheating* H) { std::memcpy(RGH_D, H, sizeof(*H) * ASTNUMFACE); }
void obtain_GPU_facet_properties(Facet_Properties* H) { std::memcpy(H, FP_D, sizeof(*H) * ASTNUMFACE); }
void obtain_GPU_roughness_shadows(Roughness_Shadow* H) { std::memcpy(H, RS_D, sizeof(*H) * ASTNUMFACE); }
void obtain_GPU_roughness_temperatures(Roughness_Temperatures* H) { std::memcpy(H, RT_D, sizeof(*H) * ASTNUMFACE); }
void obtain_GPU_roughness_illumination(Roughness_Illumination* H) { std::memcpy(H, RI_D, sizeof(*H) * ASTNUMFACE); }

void GPU_sfcpartialshadow(Roughness_Shadow* RS_H) {
    std::memcpy(RS_D, RS_H, sizeof(Roughness_Shadow) * ASTNUMFACE);
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_sfcpartialshadow(b, step);
    }
}
void GPU_single_scattering(float solar) {
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_single_scattering(b, solar, step);
    }
}
void GPU_multiple_scattering(float solar, float acc) {
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_multiple_scattering(b, solar, acc, step);
    }
}
void GPU_zero_temperatures() {
    for (int b = 0; b < ASTNUMFACE; ++b) std::memset(&RT_D[b], 0, sizeof(Roughness_Temperatures));
}
void GPU_initialise_temperatures(float EPS, float SIGMA) {
    float ES = EPS * SIGMA;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < ASTNUMFACE; ++b) k_initialise_temperatures(b, ES);
}
void GPU_inertia_difference(float EPS, float SIGMA, float TACC) {
    float ES = EPS * SIGMA, TACC2 = TACC / 10.0f;
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) { k_finite_difference(b); k_boundary_condition(b, ES, TACC2, step); }
    }
}
void GPU_inst_equilibrium(float EPS, float SIGMA) {
    float ES = EPS * SIGMA;
    for (int step = 0; step != NTAU; ++step) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < ASTNUMFACE; ++b) k_inst_equilibrium(b, ES, step);
    }
}
void GPU_converged(float TACC) {
#pragma omp parallel for schedule(static)
    for (int b = 0; b < ASTNUMFACE; ++b) k_converged(b, TACC);
}
}
#endif

namespace {
// crater geometry and the 10x10 sub-point multipliers (GPU_code.cu:611-690)
void set_constants(const GPU_Surface& S_H) {
    for (int i = 0; i != SFCNUMVTX; ++i)
        for (int k = 0; k < 3; ++k) c_vertex[i][k] = S_H.SV[i].pos[k];
    for (int j = 0; j != SFCNUMFACE; ++j) {
        for (int k = 0; k < 3; ++k) c_facet[j][k] = S_H.SF[j].sfcvertices[k];
        for (int a = 0; a < 2; ++a)
            for (int k = 0; k < 3; ++k) c_trivector[j][a][k] = S_H.SF[j].trivector[a][k];
    }
    for (int k = 1; k != m + 1; ++k)
        for (int l = 1; l != k + 1; ++l) {
            int p = ((k - 1) * (k - 1)) + (2 * (l - 1));
            c_mult[p][0] = (float)k - (1.0f / 3.0f);
            c_mult[p][1] = (float)l - (2.0f / 3.0f);
        }
    for (int k = 2; k != m + 1; ++k)
        for (int l = 1; l != k; ++l) {
            int p = ((k - 1) * (k - 1)) + (2 * (l - 1)) + 1;
            c_mult[p][0] = (float)k - (2.0f / 3.0f);
            c_mult[p][1] = (float)l - (1.0f / 3.0f);
        }
}
}  // namespace
