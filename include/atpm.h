/*
 * atpm.h -- C ABI of the GB300-native BinaryTPM thermophysical hot path.
 *
 * The reference (SamuelLeeJackson/BinaryTPM) implements its hot path as C++
 * functions over an `Asteroid&` inside one compile-time-configured program.
 * This ABI exposes the same stages as calls on an opaque solve handle, with
 * runtime sizes, caller-owned host buffers and device state owned by the
 * handle.  Each entry point names the reference function it replaces.
 *
 * Conventions
 *  - Every call returns atpm_status; nothing aborts.  atpm_last_error()
 *    returns a thread-local message for the last failure.
 *  - Host arrays are facet-major [nf][ntau], the reference's AoS order
 *    (AstFacet::_stemp[2][NTAU], 3905/Thermal/NominalPole/main.cpp:200-206).
 *  - Precision ATPM_REFERENCE evaluates every float expression of the
 *    reference CPU path in its operand order (no contraction, glibc-exact
 *    powf), so temperatures and per-revolution convergence counts are
 *    bit-identical to the reference run.  ATPM_FP64 carries the state in
 *    double.  ATPM_FAST is the batched FP32 path (contracted, BF16 view
 *    factors on the tensor cores, FP32 body-centred shadowing).
 *  - A solve handle is not thread-safe; distinct handles may be used from
 *    distinct threads.  Each handle owns one CUDA stream.
 */
#ifndef ATPM_H
#define ATPM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define ATPM_API __attribute__((visibility("default")))
#else
#define ATPM_API
#endif

typedef enum atpm_status {
    ATPM_OK = 0,
    ATPM_E_INVALID = 1,      /* bad argument or shape */
    ATPM_E_CUDA = 2,         /* a CUDA runtime call failed */
    ATPM_E_NOMEM = 3,        /* device or host allocation failed */
    ATPM_E_UNSUPPORTED = 4,  /* size or mode outside what this build handles */
    ATPM_E_STATE = 5,        /* call out of order (e.g. no forcing yet) */
    ATPM_E_NONFINITE = 6,    /* a temperature became NaN/Inf */
    ATPM_E_ITERATION = 7,    /* a device loop hit its iteration cap */
    ATPM_E_BUDGET = 8,       /* serving: request larger than the HBM budget */
    ATPM_E_CANCELLED = 9     /* serving: request cancelled */
} atpm_status;

typedef enum atpm_precision {
    ATPM_REFERENCE = 0,  /* FP32, reference operand order, bit-exact */
    ATPM_FP64 = 1,       /* plain FP64 state and arithmetic */
    ATPM_FAST = 2        /* batched FP32 + BF16 view factors */
} atpm_precision;

/* Shape model + its view-factor lists (the reference's text mesh and
 * <shape>_selfheating_list.txt, main.cpp:400-434).  dep_* is CSR:
 * row f lists the facets f sees (dep_idx) and their view factors (dep_vf),
 * in file order. */
typedef struct atpm_shape {
    int32_t nv, nf;
    const double* vertices;   /* [nv][3] km, body frame */
    const int32_t* facets;    /* [nf][3] 0-based */
    const int32_t* dep_ptr;   /* [nf+1] */
    const int32_t* dep_idx;   /* [nnz] */
    const float* dep_vf;      /* [nnz] */
} atpm_shape;

/* The reference's compile-time constants (main.cpp:17-64), at run time. */
typedef struct atpm_params {
    int32_t ntau;              /* NTAU: steps per rotation */
    int32_t nx;                /* NX: depth intervals to 8 skin depths */
    double polar[3];           /* polar0 (AU), polar1, polar2 (rad) */
    double pole[2];            /* rot0, rot1 (rad) */
    float rotation_period_s;   /* rotation_period */
    float albedo;              /* bond_albedo */
    float emissivity;          /* EPS */
    float tacc;                /* TACC (K) */
    float scattering_accuracy; /* scattering_accuracy (W/m^2) */
    int32_t shadowing;         /* 0 off, 1 view-factor list (Thermal), 2 all pairs (Visibility) */
    int32_t multiple_scattering; /* 0/1 */
    int32_t revcap;            /* revolution cap (reference: 301) */
    int32_t precision;         /* atpm_precision */
    int32_t freeze;            /* 1: converged facets stop updating (reference,
                                  main.cpp:1503); 0: every facet advances every
                                  revolution (schedule-independent comparisons) */
} atpm_params;

typedef struct atpm_context atpm_context;
typedef struct atpm_solve atpm_solve;
typedef struct atpm_crater atpm_crater;  /* crater (surface roughness) module, below */

ATPM_API const char* atpm_status_string(atpm_status s);
ATPM_API const char* atpm_last_error(void);
ATPM_API int32_t atpm_version(void);

/* Device selection + shared tables (set_cuda_device, GPU_code.cu:600-605). */
ATPM_API atpm_status atpm_context_create(int32_t device, atpm_context** out);
ATPM_API atpm_status atpm_context_destroy(atpm_context* ctx);

/* Upload a shape and allocate the solve's resident state
 * (Asteroid::Asteroid + readmodel + readselfheating, main.cpp:372-434). */
ATPM_API atpm_status atpm_solve_create(atpm_context* ctx, const atpm_shape* shape,
                                       const atpm_params* params, atpm_solve** out);
ATPM_API atpm_status atpm_solve_destroy(atpm_solve* s);
/* A new solve with the same shape, parameters and device state as `src`
 * (forcing, temperatures, convergence, tensor-core tiles), copied on the
 * device: the thermal-inertia loop of the reference's driver
 * (3905/Thermal/NominalPole/main.cpp:2481-2495) reruns one shape and forcing
 * for every thermal inertia, so a sweep uploads and prepares the shape once
 * and clones it per inertia.  No counterpart function in the reference. */
ATPM_API atpm_status atpm_solve_clone(atpm_solve* src, atpm_solve** out);
/* Device bytes held by a solve with this shape and params (HBM admission). */
ATPM_API atpm_status atpm_solve_footprint(const atpm_shape* shape, const atpm_params* params,
                                          uint64_t* bytes);

/* asteroidgeometry (main.cpp:894-1048) + astshadow (main.cpp:1286-1315, or
 * the all-pairs form of Visibility/main.cpp:674-704 when shadowing == 2). */
ATPM_API atpm_status atpm_geometry_shadow(atpm_solve* s);
/* singlescattering + multiplescattering (main.cpp:1321-1433). */
ATPM_API atpm_status atpm_scattering(atpm_solve* s);
/* Replace the forcing with caller data ([nf][ntau] shadow 0/1 and total
 * illumination W/m^2), e.g. from a reference Thermal run. */
ATPM_API atpm_status atpm_set_forcing(atpm_solve* s, const int32_t* shadow, const float* illumination);
/* Thermal inertia for the next revolutions; resets the convergence status
 * (reset_asteroid_status + the TI assignment, main.cpp:2484-2493). */
ATPM_API atpm_status atpm_set_thermal_inertia(atpm_solve* s, float ti);
/* initialisetemperatures (main.cpp:1439-1467). */
ATPM_API atpm_status atpm_initialise_temperatures(atpm_solve* s);
/* One revolution: inertiadifference (main.cpp:1473-1557) or, for TI == 0,
 * instequilibrium (main.cpp:1563-1612); then shape_converged
 * (main.cpp:1876-1909) when rev > 5.  Outputs may be NULL. */
ATPM_API atpm_status atpm_revolution(atpm_solve* s, int32_t rev, int32_t* numconverged,
                                     int32_t* converged);
/* The revolution loop of single_model (main.cpp:2521-2539): revolutions
 * until converged or revcap; counts[rev] = facets converged after rev. */
ATPM_API atpm_status atpm_run(atpm_solve* s, int32_t* nrev, int32_t* counts);
/* Whole single_model flow for a TI sweep with warm start (main.cpp:2417-2590,
 * roughness off): geometry, scattering, then per TI atpm_run.
 * nrev[nti], counts[nti][revcap]; stemp1_out (may be NULL) gets the last TI. */
ATPM_API atpm_status atpm_single_model(atpm_solve* s, const float* ti, int32_t nti, int32_t* nrev,
                                       int32_t* counts, float* stemp1_out);

/* Batched revolution loop: every solve runs atpm_run semantics, all solves
 * advance together in shared launches until each converges or hits revcap.
 * Solves must share precision and nx.  nrev[n], counts[n][revcap]. */
ATPM_API atpm_status atpm_batch_run(atpm_solve* const* solves, int32_t n, int32_t* nrev,
                                    int32_t* counts);

/* Host copies of the solve's state ([nf][ntau] facet-major). */
/* A solve's Bond albedo (the reference's bond_albedo, main.cpp:38), e.g. for a
 * clone that shares its source's shape and shadows: the scattered
 * illumination depends on it, so atpm_scattering runs again before the
 * next revolution. */
ATPM_API atpm_status atpm_set_albedo(atpm_solve* s, float albedo);
/* the solar flux at the body (A.rtnsolar(), main.cpp:905), W/m^2 */
ATPM_API atpm_status atpm_solve_solar(const atpm_solve* s, float* solar);
ATPM_API atpm_status atpm_get_shadow(atpm_solve* s, int32_t* out);
ATPM_API atpm_status atpm_get_illumination(atpm_solve* s, float* out);
ATPM_API atpm_status atpm_get_surface_temperature(atpm_solve* s, float* stemp1, float* stemp0);
ATPM_API atpm_status atpm_get_surface_temperature64(atpm_solve* s, double* stemp1);
/* The Thermal stage's result of n solves at once: stemp1[i] receives solve
 * i's surface temperatures as atpm_get_surface_temperature does ([nf][ntau]
 * FP32).  Each solve's transpose and copy run on its own stream, so the
 * copies to the host overlap; the call returns when all have landed. */
ATPM_API atpm_status atpm_get_surface_temperatures(atpm_solve* const* solves, int32_t n, float* const* stemp1);
ATPM_API atpm_status atpm_get_depth_temperature(atpm_solve* s, float* temp /* [nf][nx+1] */);
/* (float)cos of the Sun angle of every facet and step ([nf][ntau]). */
ATPM_API atpm_status atpm_get_cosillum(atpm_solve* s, float* out);
/* Per-facet convergence flags after the last revolution, 1 = converged (and
 * frozen when the solve freezes): the facet property _astconverged
 * (3905/Thermal/NominalPole/main.cpp:193, 303). */
ATPM_API atpm_status atpm_get_converged(atpm_solve* s, uint8_t* out /* [nf] */);
/* One revolution of the given (active) solves with a CUDA event between
 * kernels: kernel_ms[5] = self-heating W, self-heating Q, conduction,
 * convergence, advance.  Advances the solves by one revolution. */
ATPM_API atpm_status atpm_profile_revolution(atpm_solve* const* solves, int32_t n, double* kernel_ms,
                                             int64_t* facet_steps, int64_t* active_facets);
/* Self-heating flux Q[s][f] = sum_g V[f][g] eps sigma T_g[s]^4 for the
 * current surface temperatures ([ntau][nf] step-major), through the solve's
 * own path (list-order gather, or the BF16 tensor-core product for FAST),
 * for every facet, frozen ones included. */
ATPM_API atpm_status atpm_selfheating_flux(atpm_solve* s, float* q);
/* Non-synchronous binary (the 175706 Thermal program,
 * 175706/Run-04/thermal.cpp:1347-1381, 860-869, 1925-1967): the first
 * primary_vertices vertices and primary_facets facets form the primary,
 * which turns primary_revs times during the model period (params.ntau steps
 * over params.rotation_period_s); the other vertices and facets (the
 * secondary, turning about the same axis) turn secondary_revs times.  Each
 * body's conduction uses its own time step and skin-depth factor.  Mutual
 * eclipses need all-pairs shadowing (params.shadowing = 2).  Call before
 * atpm_geometry_shadow. */
ATPM_API atpm_status atpm_set_binary_rotation(atpm_solve* s, int32_t primary_vertices, int32_t primary_facets,
                                              int32_t primary_revs, int32_t secondary_revs);
/* IR absorptivity applied to the self-heating sum (IR_ABS,
 * 175706/Run-04/thermal.cpp:72, 1950-1952); 1 unless set. */
ATPM_API atpm_status atpm_set_ir_absorptivity(atpm_solve* s, float ir_abs);
/* Orbital sweeps (orbital_model / obliquity_model, main.cpp:2612-3003): the
 * heliocentric body centre (km) at true anomaly ta_deg of a Keplerian orbit
 * (orbital_position_geometry, main.cpp:800-810), and a solve placed there
 * instead of at params.polar (heliocentric distance and solar constant
 * follow, main.cpp:901-905).  Call atpm_set_position before
 * atpm_geometry_shadow; solves at different orbital points (or poles) batch
 * together in atpm_batch_run. */
ATPM_API atpm_status atpm_orbital_position(double a_au, double e, double inc_deg, double node_deg, double peri_deg,
                                           double ta_deg, double* car_km);
ATPM_API atpm_status atpm_set_position(atpm_solve* s, const double* car_km);
/* Disk-integrated thermal flux seen by an observer, FP64 on the device: the
 * smooth-surface sum of the Observe stage's observe
 * (3905/Observe/NominalPole/wise_main.cpp:662-730, its geometry 555-645).
 * observer: the body's position as seen by the observer (distance in AU,
 * ecliptic latitude, longitude in rad: the stage's obs_polar0..2,
 * wise_main.cpp:27-29); the body is at the solve's polar; observer = polar
 * means seen from the Sun (zero phase).  Like the stage, positions are in
 * metres (its AU = 149.6e9 m) while the shape keeps its own units;
 * visibility: [nf][ntau] flags toward the observer (the Visibility stage's
 * output, e.g. atpm_get_shadow of a solve with the observer as polar and
 * shadowing 2), or NULL for each facet's own horizon test only; wavelengths
 * emissivity: the stage's double EPS (wise_main.cpp:13); wavelengths in
 * micrometres (1..8 of them); flux: [ntau][nwl], Planck radiance times
 * eps * area * cos(e) / distance^2.  Uses the
 * solve's current surface temperatures; facet sums run in a fixed order
 * (deterministic). */
ATPM_API atpm_status atpm_disk_flux(atpm_solve* s, const double* observer, const int32_t* visibility,
                                    double emissivity, int32_t nwl, const double* wavelength_um, double* flux);
/* The rough-surface sum of the same stage (observe, wise_main.cpp:695-727),
 * FP64 on the device, for the fitting's roughness mix R * rough +
 * (1 - R) * smooth (175706/Run-04/fitting.cpp:460-461): every facet visible
 * at a step contributes its crater's sub-facets with a visible fraction > 0,
 * B(T_sub) * eps * a_sub * vis_sub * cos(e_sub) / d^2, the facet's total
 * scaled by its area over the crater's projected area sum(a_sub * n_sub,z).
 * temperatures: a crater (atpm_crater_create with nx > 0) holding the
 * sub-facet surface temperatures of this solve's facets (its stemp1);
 * sub_visibility: a crater whose sub-facet shadow array (set/get_array 1)
 * holds each sub-facet's visible fraction toward the observer (the
 * Visibility stage's crater output: a crater shadow run with the observer
 * as the light source); crater_vertices [nsv][3] float and crater_facets
 * [nsf][3]: the crater model as the stage reads it from the roughness
 * visibility file.  Other arguments as atpm_disk_flux; flux [ntau][nwl].
 * The stage computes this sum in the loop of atpm_disk_flux's. */
ATPM_API atpm_status atpm_disk_flux_rough(atpm_solve* s, const atpm_crater* temperatures,
                                          const atpm_crater* sub_visibility, int32_t nsv, const float* crater_vertices,
                                          const int32_t* crater_facets, const double* observer,
                                          const int32_t* visibility, double emissivity, int32_t nwl,
                                          const double* wavelength_um, double* flux);
/* FP64 diagnostics of the last revolution: sum over facets and steps of the
 * absorbed flux, emitted flux and the mean surface temperature. */
ATPM_API atpm_status atpm_energy_balance(atpm_solve* s, double* absorbed, double* emitted,
                                         double* mean_temperature);
/* Failure-path self-test of the bounded waits: a one-thread kernel waits on
 * an mbarrier that nothing arrives at, with the bounded wait every pipeline
 * wait of the tensor-core product uses (limit_cycles clock cycles, at most
 * ~1 s), records ST_TC_TIMEOUT (16) in status_bits and returns.  Returns
 * ATPM_E_ITERATION when the wait gave up (the expected outcome) and leaves
 * the device context usable.  No copy, product or TMEM allocation runs.
 * No counterpart in the reference, whose kernels have no bounded waits. */
ATPM_API atpm_status atpm_selftest_bounded_wait(int32_t device, int64_t limit_cycles, int32_t* status_bits);
/* The shadow drivers of the last atpm_geometry_shadow: their device time
 * (ms, CUDA events), the rays they answered (facet x step queries: is this
 * facet's midpoint occluded toward the Sun or observer at this step) and the
 * exact ray-triangle tests (astshadowtest, main.cpp:1187-1247) the culled
 * drivers ran after their box tests; exact_tests is -1 when the plain
 * drivers ran (ATPM_SHADOW_CULL=0). */
ATPM_API atpm_status atpm_last_shadow_stats(atpm_solve* s, double* shadow_ms, int64_t* rays, int64_t* exact_tests);
/* Launch configuration of the last atpm_batch_run led by s (FAST): the
 * conduction register/occupancy variant (1-3), the tensor-core pipeline
 * depth, and whether that run timed the candidates (the autotuner does so
 * on the first three revolutions of the first batch of each kind; its
 * choices never change results).  ATPM_AUTOTUNE=0 turns it off. */
ATPM_API atpm_status atpm_last_run_config(atpm_solve* s, int32_t* cond_variant, int32_t* tc_stages, int32_t* tuned);
/* Device time (ms, CUDA events on the solve's stream) of the last atpm_run /
 * atpm_batch_run revolution loop, and launches issued inside it. */
ATPM_API atpm_status atpm_last_run_stats(atpm_solve* s, double* device_ms, int64_t* launches,
                                         int64_t* facet_steps);

/* ---- view factors: the Shape_Selfheating stage (3905/Shape_Selfheating/main.cpp:817-889) ----
 * Facing screen + view factor of every facet pair (selfheating, main.cpp:628-744),
 * occlusion culling over each facet's candidate list (hidden, main.cpp:187-368)
 * and, when refine != 0, 10x10 sub-facet refinement of pairs with vf >= 0.05
 * (betterviewfactors, main.cpp:374-622).  Vertices are float like the
 * reference's reader.  The result is held until atpm_viewfactors_free. */
typedef struct atpm_vf_result atpm_vf_result;
ATPM_API atpm_status atpm_viewfactors_compute(atpm_context* ctx, int32_t nv, int32_t nf, const float* vertices,
                                              const int32_t* facets, int32_t refine, atpm_vf_result** out,
                                              int64_t* nnz);
/* dep_ptr[nf+1], dep_idx[nnz], dep_vf[nnz], dep_vec[nnz][3] (area-weighted
 * direction sums, main.cpp:730-732 and 592-602), photovectors[nf][3]
 * (main.cpp:824-835); any output may be NULL. */
ATPM_API atpm_status atpm_viewfactors_get(const atpm_vf_result* r, int32_t* dep_ptr, int32_t* dep_idx, float* dep_vf,
                                          float* dep_vec, float* photovectors);
ATPM_API atpm_status atpm_viewfactors_free(atpm_vf_result* r);

/* ---- crater (surface roughness) module ----
 * Runtime-sized counterpart of the reference's Thermal GPU module
 * (3905/Thermal/NominalPole/GPU_code.cu:600-1026).  Arrays are
 * [facet][step][sub-facet] like the module's structs; nsf = crater
 * sub-facets (100 for the shipped crater).  REFERENCE precision follows the
 * module's float expressions operand by operand (no contraction, this host's
 * libm powf), FAST contracts. */
/* initialise_GPU_*_arrays (GPU_code.cu:696-768).  nx = 0 creates a
 * shadow-only crater (the Visibility stage's module,
 * 3905/Visibility/NominalPole/GPU_code.cu:146-283): only the shadow arrays
 * (set/get_array 0-3) are held, the thermal calls return ATPM_E_STATE. */
ATPM_API atpm_status atpm_crater_create(atpm_context* ctx, int32_t nf, int32_t ntau, int32_t nx, int32_t nsf,
                                        int32_t precision, atpm_crater** out);
/* freeup_GPU_*_arrays (774-812) */
ATPM_API atpm_status atpm_crater_destroy(atpm_crater* c);
/* initialise_GPU_constants (611-690): crater vertices [nsv][3], facets
 * [nsf][3], sub-triangle vectors [nsf][2][3], view factors V[i][j] [nsf][nsf]
 * (may be NULL for a shadow-only crater) */
ATPM_API atpm_status atpm_crater_set_model(atpm_crater* c, int32_t nsv, const float* vertices, const int32_t* facets,
                                           const float* trivectors, const float* viewfactors, float rot_period);
/* set_GPU_facet_properties / obtain_GPU_facet_properties (818-825, 857-863) */
ATPM_API atpm_status atpm_crater_set_properties(atpm_crater* c, const uint8_t* converged, const float* albedo,
                                                const float* thermal_inertia);
ATPM_API atpm_status atpm_crater_get_properties(atpm_crater* c, uint8_t* converged, float* albedo,
                                                float* thermal_inertia);
/* which: 0 facet shadow (int32 [nf][ntau]), 1 sub-facet shadow, 2 crater Sun
 * vector ([nf][ntau][3]), 3 sub-facet Sun angle, 4 illumination, 5 global
 * illumination, 6 global heating ([nf][ntau][nsf] floats) -- the fields of
 * Roughness_Shadow / Illumination / Globalillumination / Globalheating
 * (GPU_code.cu:85-124; load_GPU_* 831-851, obtain_GPU_* 866-903) */
ATPM_API atpm_status atpm_crater_set_array(atpm_crater* c, int32_t which, const void* data);
ATPM_API atpm_status atpm_crater_get_array(atpm_crater* c, int32_t which, void* data);
/* The same transfers straight from / into an array of per-facet structs:
 * facet f's block of array `which` starts at base + f * facet_stride bytes
 * (the module's AoS layout: pass the field's address in element 0 and
 * sizeof the struct).  which 7, 8, 9 are stemp0, stemp1 ([nf][ntau][nsf]) and
 * the depth columns ([nf][nx+1][nsf]) of Roughness_Temperatures.  One strided
 * copy each way, no host-side repacking. */
ATPM_API atpm_status atpm_crater_set_array_strided(atpm_crater* c, int32_t which, const void* base,
                                                   uint64_t facet_stride);
ATPM_API atpm_status atpm_crater_get_array_strided(atpm_crater* c, int32_t which, void* base, uint64_t facet_stride);
/* Non-synchronous binaries (the 175706 program's module,
 * 175706/Run-04/thermal_GPU.cu): each facet's body turns numrevs[f] times
 * per model period, which scales that facet's crater time step and skin
 * factor (thermal_GPU.cu:448-450, 539); NULL returns every facet to one
 * turn, the synchronous module's expressions.  The IR absorptivity scales
 * the crater sub-facets' emission seen by the others (thermal_GPU.cu:521,
 * 390, 615); 1 unless set. */
ATPM_API atpm_status atpm_crater_set_revolutions(atpm_crater* c, const float* numrevs /* [nf] or NULL */);
/* The crater model from its mesh alone (the shim path gets the derived
 * vectors from the driver instead): vertices [nsv][3], facets [nsf][3] and
 * view factors V[i][j] as for atpm_crater_set_model; the sub-point grid
 * vectors and the sub-facet unit normals are derived as surfacegeometry does
 * (3905/Thermal/NominalPole/main.cpp:822-868).  Needed by atpm_crater_forcing. */
ATPM_API atpm_status atpm_crater_set_surface(atpm_crater* c, int32_t nsv, const float* vertices,
                                             const int32_t* facets, const float* viewfactors, float rot_period);
/* The crater's forcing for facets f0 .. f0 + nf - 1 of a solve (a part, in
 * the reference's terms), computed on the device from the solve's geometry,
 * shadows and scattered illumination (after atpm_geometry_shadow and
 * atpm_scattering; REFERENCE or FAST solves): the facet shadows and local
 * Sun vectors (asteroidgeometry, main.cpp:1019-1030), each sub-facet's Sun
 * angle and starting shadow (surfacegeometry, 873-885), the sub-facet view
 * factors of the solve's list entries (calculate_surface_global_viewfactors,
 * 1053-1181) and the global illumination (2033-2065) -- arrays 0-3 and 5.
 * dep_vec: the solve's list entries' direction vectors [nnz][3] (the
 * _selfheating_vector_list.txt vectors; NULL when the part has no entries).
 * A REFERENCE crater on a REFERENCE solve gives the arrays the reference
 * driver builds on the host, bit for bit. */
ATPM_API atpm_status atpm_crater_forcing(atpm_solve* s, atpm_crater* c, int32_t f0, const float* dep_vec);
/* The global heating (array 6) from the solve's current surface temperatures
 * (load_GPU_roughness_globalheating, main.cpp:2069-2103), with the view
 * factors of the last atpm_crater_forcing on the same solve and f0. */
ATPM_API atpm_status atpm_crater_global_heating(atpm_solve* s, atpm_crater* c, int32_t f0);
/* One crater for parts of several solves (rough solves of a batch sharing
 * the crater launches): facets f0 .. f0 + n - 1 of solve s go to facets
 * c0 .. c0 + n - 1 of the crater, whose forcing (as atpm_crater_forcing) and
 * global heating from the solve's current surface temperatures (as
 * atpm_crater_global_heating) are computed for that range alone.  Each
 * facet keeps its own thermal inertia and albedo (atpm_crater_set_properties);
 * the parts share NTAU, NX, the crater model, its rotation period and the
 * solar flux given to atpm_crater_scattering.  The crater revolutions then
 * advance every part in the same launches, each facet's columns exactly as
 * in a crater of that part alone. */
ATPM_API atpm_status atpm_crater_prepare_part(atpm_solve* s, atpm_crater* c, int32_t f0, int32_t c0, int32_t n,
                                              const float* dep_vec);
ATPM_API atpm_status atpm_crater_set_ir_absorptivity(atpm_crater* c, float ir_abs);
/* GPU_sfcpartialshadow (909-921): every step in one launch */
ATPM_API atpm_status atpm_crater_partial_shadow(atpm_crater* c);
/* GPU_single_scattering / GPU_multiple_scattering (927-949) */
ATPM_API atpm_status atpm_crater_scattering(atpm_crater* c, float solar, float accuracy, int32_t multiple);
/* GPU_zero_temperatures / GPU_initialise_temperatures (955-976) */
ATPM_API atpm_status atpm_crater_zero_temperatures(atpm_crater* c);
ATPM_API atpm_status atpm_crater_initialise_temperatures(atpm_crater* c, float eps, float sigma);
/* GPU_inertia_difference (982-998): one revolution, one launch */
ATPM_API atpm_status atpm_crater_inertia_difference(atpm_crater* c, float eps, float sigma, float tacc);
/* GPU_inst_equilibrium (1004-1015) */
ATPM_API atpm_status atpm_crater_inst_equilibrium(atpm_crater* c, float eps, float sigma);
/* GPU_converged (1021-1026) */
ATPM_API atpm_status atpm_crater_converged(atpm_crater* c, float tacc);
/* obtain_GPU_roughness_temperatures (879-886): [nf][ntau][nsf], temp [nf][nx+1][nsf] */
ATPM_API atpm_status atpm_crater_get_temperatures(atpm_crater* c, float* stemp0, float* stemp1, float* temp);

/* ---- serving: continuous batching on one GPU ----
 * A server keeps many solves resident and advances them together: shapes
 * are registered once (geometry, shadowing and scattering computed and kept
 * on the device), requests carry a thermal inertia, are admitted while a
 * batch slot is free and their device footprint fits the HBM budget, and
 * every scheduler tick advances all resident solves by revs_per_tick
 * revolutions in shared launches.  Finished solves are retired (results
 * copied out, memory returned) and waiting requests admitted in their place.
 * A result does not depend on what else was in the batch. */
typedef struct atpm_server atpm_server;
ATPM_API atpm_status atpm_server_create(atpm_context* ctx, int32_t precision, int32_t nx, uint64_t budget_bytes,
                                        int32_t max_active, int32_t revs_per_tick, atpm_server** out);
ATPM_API atpm_status atpm_server_add_shape(atpm_server* s, const atpm_shape* shape, const atpm_params* params,
                                           int32_t* shape_id);
ATPM_API atpm_status atpm_server_submit(atpm_server* s, int32_t shape_id, float thermal_inertia, int64_t* request_id);
ATPM_API atpm_status atpm_server_cancel(atpm_server* s, int64_t request_id);
/* Wait up to timeout_s for a request; stemp1 [nf][ntau] (may be NULL).  A
 * wait that finds the request finished hands its result over and forgets
 * the request (a later wait on the same id is ATPM_E_INVALID); a wait that
 * times out (ATPM_E_STATE) leaves it to a later wait. */
ATPM_API atpm_status atpm_server_wait(atpm_server* s, int64_t request_id, double timeout_s, float* stemp1,
                                      int32_t* nrev, double* latency_s);
/* Latency percentiles (submit to result) and facet-steps/s of completed requests. */
ATPM_API atpm_status atpm_server_stats(atpm_server* s, double* p50_s, double* p99_s, double* facet_steps_per_s,
                                       int64_t* completed, uint64_t* resident_bytes);
ATPM_API atpm_status atpm_server_destroy(atpm_server* s);

/* ---- no device allocation ----
 * Single + multiple scattering (the computation of atpm_scattering) over
 * caller-owned DEVICE buffers, allocating nothing: for callers that cannot
 * allocate device memory (a framework that owns every allocation through its
 * own pool, or code that must not trigger allocator synchronisation).  The
 * Gauss-Seidel work arrays live in one fixed file-scope device array of
 * 2^20 cells x 3 floats (12 MiB), reserved on every GPU that loads the
 * library until exit.  No counterpart in the reference.
 *   nf * ntau must be <= 2^20 and nf <= 524,280, otherwise
 *   ATPM_E_UNSUPPORTED.
 *   dep_ptr/idx/vf: CSR lists, all three device pointers (never NULL, even
 *   for empty lists); cosillum [nf][ntau] float; shadow [nf][ntau] bytes
 *   0/1; illumination [nf][ntau] float output.  status: device int the
 *   kernels OR ST_* bits into (8 = scattering cap reached: Gauss-Seidel
 *   stopped at 1,000 sweeps); the caller zeroes it.  It is required when
 *   multiple != 0 (ATPM_E_INVALID otherwise) and may be NULL for single
 *   scattering only.  Work is enqueued on `stream` (a cudaStream_t,
 *   NULL = default stream); the call returns without waiting for it.
 *   The first call on a device looks up the array's address
 *   (cudaGetSymbolAddress) with that device current: make it before any
 *   stream capture on that device.  Calls share the array: calls that
 *   overlap on the GPU race and must be serialised by the caller. */
ATPM_API atpm_status atpm_scattering_noalloc(int32_t nf, int32_t ntau, const int32_t* dep_ptr, const int32_t* dep_idx,
                                             const float* dep_vf, const float* cosillum, const uint8_t* shadow,
                                             float solar, float albedo, float scattering_accuracy, int32_t multiple,
                                             float* illumination, int32_t* status, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ATPM_H */
