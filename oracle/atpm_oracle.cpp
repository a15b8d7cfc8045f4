// CPU oracle for the BinaryTPM thermophysical hot path.  TEST INFRASTRUCTURE
// ONLY: tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it
// (via ctypes) to check the CUDA library; the product never calls it.
//
// It restates, with runtime sizes instead of compile-time constants, the
// smooth-shape path of the reference Thermal driver
// (3905/Thermal/NominalPole/main.cpp) and the all-pairs shadowing of the
// reference Visibility driver (3905/Visibility/NominalPole/main.cpp):
//
//   geometry            main.cpp:894-1048   asteroidgeometry
//   shadow predicate    main.cpp:1187-1247  astshadowtest
//   dependent shadowing main.cpp:1286-1315  astshadow (view-factor list)
//   all-pairs shadowing Visibility/main.cpp:674-704
//   single scattering   main.cpp:1321-1345
//   multiple scattering main.cpp:1351-1433  (Gauss-Seidel, facet order)
//   initial temperature main.cpp:1439-1467
//   conduction + BC     main.cpp:1473-1557  inertiadifference
//   TI = 0 equilibrium  main.cpp:1563-1612  instequilibrium
//   convergence         main.cpp:1876-1909  shape_converged
//   driver loop         main.cpp:2417-2590  single_model (TI sweep, rev < 301)
//
// precision 0 ("reference"): every float expression is evaluated in the
// reference's operand order with glibc powf, so with -ffp-contract=off the
// results are bit-identical to the reference binary built the same way.
// precision 1 ("fp64"): the thermal/scattering state is double and x^4 is
// (x*x)*(x*x); this is the FP64 accuracy oracle.
//
// The self-heating flux of inertiadifference reads each neighbour's
// previous-revolution surface temperature (stemp0 after it has operated in
// this step, stemp1 before: both hold the value from revolution r-1,
// main.cpp:1505-1527); the restatement reads a per-step snapshot, which is the
// race-free form of the same rule.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

namespace {

const double PI = 4.0 * std::atan(1.0);  // main.cpp:12
const double AU = 149.6e6;               // main.cpp:13
const float SIGMA = 5.67e-8f;            // main.cpp:15

}  // namespace

extern "C" {

struct oracle_params {
    int nv, nf, ntau, nx;
    const double* vertices;  // [nv][3] km, body frame
    const int32_t* facets;   // [nf][3]
    const int32_t* dep_ptr;  // [nf+1] CSR row pointers of the view-factor lists
    const int32_t* dep_idx;  // [nnz]
    const float* dep_vf;     // [nnz]
    double polar0, polar1, polar2;  // heliocentric distance (AU), latitude, longitude (rad)
    double rot0, rot1;              // pole latitude, longitude (rad)
    float tacc, scattering_accuracy, eps, rotation_period, albedo;
    int shadowing;            // 0 off, 1 dependent-list (Thermal), 2 all-pairs (Visibility)
    int multiple_scattering;  // 0/1
    int precision;            // 0 reference float, 1 fp64
    int revcap;               // reference: 301
    int nti;
    const float* ti;          // [nti] thermal inertia sweep (warm-started, main.cpp:2481-2517)
    int nthreads;
};

struct oracle_outputs {
    int32_t* shadow;      // [nf][ntau]
    float* illumination;  // [nf][ntau] total illumination after scattering
    float* cosillum;      // [nf][ntau] (float)cos(illumangle)
    double* illumination64;  // [nf][ntau] (precision 1 only, may be null)
    float* stemp1;        // [nf][ntau] final surface temperature of the last TI
    float* stemp0;        // [nf][ntau]
    float* temp;          // [nf][nx+1]
    double* stemp1_64;    // [nf][ntau] (precision 1 only, may be null)
    int32_t* numconverged;  // [nti][revcap]
    int32_t* nrev;        // [nti]
};

}  // extern "C"

namespace {

struct Geometry {
    int nv, nf, ntau;
    std::vector<double> heliopos;     // [ntau][nv][3]
    std::vector<double> heliomidpos;  // [ntau][nf][3]
    std::vector<double> normal;       // [ntau][nf][3]
    std::vector<double> illumangle;   // [nf][ntau]
    std::vector<int32_t> shadow;      // [nf][ntau]
    float solar;
};

// main.cpp:894-1048 (single_run == 1 branch)
void asteroidgeometry(const oracle_params& P, Geometry& G) {
    const int nv = P.nv, nf = P.nf, ntau = P.ntau;
    G.nv = nv; G.nf = nf; G.ntau = ntau;
    G.heliopos.assign((size_t)ntau * nv * 3, 0.0);
    G.heliomidpos.assign((size_t)ntau * nf * 3, 0.0);
    G.normal.assign((size_t)ntau * nf * 3, 0.0);
    G.illumangle.assign((size_t)nf * ntau, 0.0);
    G.shadow.assign((size_t)nf * ntau, 1);
    double carcentre[3];
    carcentre[0] = AU * P.polar0 * cos(P.polar1) * cos(P.polar2);
    carcentre[1] = AU * P.polar0 * cos(P.polar1) * sin(P.polar2);
    carcentre[2] = AU * P.polar0 * sin(P.polar1);
    G.solar = (float)(1367.0 / (P.polar0 * P.polar0));
    const double r0 = P.rot0, r1 = P.rot1;
    double gamma = acos(cos(r0) * sin(fabs(r1)));
    double tm[3][3];
    tm[0][0] = sin(r0) / sin(gamma);
    tm[0][1] = -1.0 * cos(r0) * cos(r0) * sin(r1) * cos(r1) / sin(gamma);
    tm[0][2] = cos(r0) * cos(r1);
    tm[1][0] = 0.0;
    tm[1][1] = ((sin(r0) * sin(r0)) + (cos(r0) * cos(r0) * cos(r1) * cos(r1))) / sin(gamma);
    tm[1][2] = cos(r0) * sin(r1);
    tm[2][0] = -1.0 * cos(r0) * cos(r1) / sin(gamma);
    tm[2][1] = -1.0 * sin(r0) * cos(r0) * sin(r1) / sin(gamma);
    tm[2][2] = sin(r0);

#pragma omp parallel for schedule(dynamic) num_threads(P.nthreads)
    for (int step = 0; step < ntau; step++) {
        double rotangle = 2.0 * PI * step / ntau;
        double* hp = &G.heliopos[(size_t)step * nv * 3];
        for (int b = 0; b < nv; ++b) {
            const double* e = &P.vertices[3 * b];
            double rq[3], ec[3];
            rq[0] = (e[0] * cos(rotangle)) - (e[1] * sin(rotangle));
            rq[1] = (e[0] * sin(rotangle)) + (e[1] * cos(rotangle));
            rq[2] = e[2];
            for (int k = 0; k < 3; ++k) ec[k] = (tm[k][0] * rq[0]) + (tm[k][1] * rq[1]) + (tm[k][2] * rq[2]);
            for (int k = 0; k < 3; ++k) hp[3 * b + k] = carcentre[k] + ec[k];
        }
        for (int c = 0; c < nf; ++c) {
            const int32_t* v = &P.facets[3 * c];
            const double *h0 = &hp[3 * v[0]], *h1 = &hp[3 * v[1]], *h2 = &hp[3 * v[2]];
            double* hm = &G.heliomidpos[((size_t)step * nf + c) * 3];
            double* n = &G.normal[((size_t)step * nf + c) * 3];
            for (int k = 0; k < 3; ++k) hm[k] = ((h0[k] + h1[k]) + h2[k]) / 3.0;
            double t = sqrt((hm[0] * hm[0]) + (hm[1] * hm[1]) + (hm[2] * hm[2]));
            double nc0[3], nc1[3];
            for (int k = 0; k < 3; ++k) { nc0[k] = h1[k] - h0[k]; nc1[k] = h2[k] - h0[k]; }
            n[0] = (nc0[1] * nc1[2]) - (nc0[2] * nc1[1]);
            n[1] = (nc0[2] * nc1[0]) - (nc0[0] * nc1[2]);
            n[2] = (nc0[0] * nc1[1]) - (nc0[1] * nc1[0]);
            double nn = sqrt((n[0] * n[0]) + (n[1] * n[1]) + (n[2] * n[2]));
            n[0] = n[0] / nn; n[1] = n[1] / nn; n[2] = n[2] / nn;
            // illumvector[2] = -(normal . heliomidpos) (row 2 of imatrix is the normal)
            double iv2 = -1.0 * ((n[0] * hm[0]) + (n[1] * hm[1]) + (n[2] * hm[2]));
            double ia = acos(iv2 / t);
            G.illumangle[(size_t)c * ntau + step] = ia;
            if (ia > (PI / 2.0)) G.shadow[(size_t)c * ntau + step] = 0;
        }
    }
}

inline double norm3(const double* a) { return sqrt((a[0] * a[0]) + (a[1] * a[1]) + (a[2] * a[2])); }

// main.cpp:1187-1247.  Returns 0 when H blocks the Sun ray through G's midpoint.
int astshadowtest(const oracle_params& P, const Geometry& G, int g, int h, int step) {
    const int nf = G.nf, nv = G.nv;
    const double* Gm = &G.heliomidpos[((size_t)step * nf + g) * 3];
    const double* Hm = &G.heliomidpos[((size_t)step * nf + h) * 3];
    const double* Hn = &G.normal[((size_t)step * nf + h) * 3];
    const double* hp = &G.heliopos[(size_t)step * nv * 3];
    const int32_t* hv = &P.facets[3 * h];
    const double *V0 = &hp[3 * hv[0]], *V1 = &hp[3 * hv[1]], *V2 = &hp[3 * hv[2]];
    double tcalc2 = (Gm[0] * Hn[0]) + (Gm[1] * Hn[1]) + (Gm[2] * Hn[2]);
    double tcalc1 = (Hm[0] * Hn[0]) + (Hm[1] * Hn[1]) + (Hm[2] * Hn[2]);
    double t = tcalc1 / tcalc2;
    double x[3] = {t * Gm[0], t * Gm[1], t * Gm[2]};
    double n1[3], n2[3], n3[3], x1[3], x2[3], x3[3];
    for (int k = 0; k < 3; ++k) {
        n1[k] = V1[k] - V0[k];
        n2[k] = V0[k] - V2[k];
        n3[k] = V2[k] - V1[k];
        x1[k] = x[k] - V0[k];
        x3[k] = x[k] - V1[k];
        x2[k] = x[k] - V2[k];
    }
    double t1[3], t2[3], t3[3];
    t1[0] = (n1[1] * x1[2]) - (n1[2] * x1[1]);
    t1[1] = (n1[2] * x1[0]) - (n1[0] * x1[2]);
    t1[2] = (n1[0] * x1[1]) - (n1[1] * x1[0]);
    t2[0] = (n2[1] * x2[2]) - (n2[2] * x2[1]);
    t2[1] = (n2[2] * x2[0]) - (n2[0] * x2[2]);
    t2[2] = (n2[0] * x2[1]) - (n2[1] * x2[0]);
    t3[0] = (n3[1] * x3[2]) - (n3[2] * x3[1]);
    t3[1] = (n3[2] * x3[0]) - (n3[0] * x3[2]);
    t3[2] = (n3[0] * x3[1]) - (n3[1] * x3[0]);
    double c1 = (t1[0] * Hn[0]) + (t1[1] * Hn[1]) + (t1[2] * Hn[2]);
    double c2 = (t2[0] * Hn[0]) + (t2[1] * Hn[1]) + (t2[2] * Hn[2]);
    double c3 = (t3[0] * Hn[0]) + (t3[1] * Hn[1]) + (t3[2] * Hn[2]);
    if (c1 >= 0.0 && c2 >= 0.0 && c3 >= 0.0) return 0;
    return 1;
}

// main.cpp:1286-1315
void astshadow_deplist(const oracle_params& P, Geometry& G, int step) {
    for (int g = 0; g < G.nf; ++g) {
        const int d0 = P.dep_ptr[g], d1 = P.dep_ptr[g + 1];
        if (d1 != d0 && G.shadow[(size_t)g * G.ntau + step] == 1) {
            double gd = norm3(&G.heliomidpos[((size_t)step * G.nf + g) * 3]);
            for (int k = d0; k < d1; ++k) {
                int h = P.dep_idx[k];
                double hd = norm3(&G.heliomidpos[((size_t)step * G.nf + h) * 3]);
                if (gd > hd) {
                    if (astshadowtest(P, G, g, h, step) == 0) G.shadow[(size_t)g * G.ntau + step] = 0;
                }
            }
        }
    }
}

// 3905/Visibility/NominalPole/main.cpp:674-704
void astshadow_allpairs(const oracle_params& P, Geometry& G, int step) {
    for (int g = 0; g < G.nf; ++g) {
        double gd = norm3(&G.heliomidpos[((size_t)step * G.nf + g) * 3]);
        for (int h = g + 1; h < G.nf; ++h) {
            double hd = norm3(&G.heliomidpos[((size_t)step * G.nf + h) * 3]);
            if (gd > hd) {
                if (G.shadow[(size_t)g * G.ntau + step] == 1)
                    if (astshadowtest(P, G, g, h, step) == 0) G.shadow[(size_t)g * G.ntau + step] = 0;
            } else {
                if (G.shadow[(size_t)h * G.ntau + step] == 1)
                    if (astshadowtest(P, G, h, g, step) == 0) G.shadow[(size_t)h * G.ntau + step] = 0;
            }
        }
    }
}

template <class R> struct Real;
template <> struct Real<float> {
    static float pw4(float x) { return std::pow(x, 4.0f); }   // glibc powf, as main.cpp:1523
    static float pw3(float x) { return std::pow(x, 3.0f); }   // main.cpp:1538
    static float pwq(float x) { return std::pow(x, 0.25f); }  // main.cpp:1458
    static float cosv(double a) { return (float)cos(a); }     // main.cpp:1331
};
template <> struct Real<double> {
    static double pw4(double x) { double t2 = x * x; return t2 * t2; }
    static double pw3(double x) { return (x * x) * x; }
    // FP64 mode defines x^0.25 as two correctly rounded square roots (the
    // GPU's FP64 path evaluates the same expression)
    static double pwq(double x) { return std::sqrt(std::sqrt(x)); }
    static double cosv(double a) { return cos(a); }
};

template <class R>
struct Thermal {
    const oracle_params& P;
    const Geometry& G;
    int nf, ntau, nx;
    std::vector<R> illum;   // [nf][ntau]
    std::vector<R> stemp0, stemp1;  // [nf][ntau]
    std::vector<R> temp;    // [nf][nx+1]
    std::vector<uint8_t> conv;
    int numconverged = 0, converged = 0;

    Thermal(const oracle_params& p, const Geometry& g) : P(p), G(g), nf(p.nf), ntau(p.ntau), nx(p.nx) {
        illum.assign((size_t)nf * ntau, R(0));
        stemp0.assign((size_t)nf * ntau, R(0));
        stemp1.assign((size_t)nf * ntau, R(0));
        temp.assign((size_t)nf * (nx + 1), R(0));
        conv.assign(nf, 0);
    }

    R shadowf(int f, int s) const { return (R)G.shadow[(size_t)f * ntau + s]; }
    R cosf_(int f, int s) const { return Real<R>::cosv(G.illumangle[(size_t)f * ntau + s]); }

    // main.cpp:1321-1345
    void singlescattering() {
        const R solar = (R)G.solar;
        const R alb = (R)P.albedo;
#pragma omp parallel for schedule(dynamic) num_threads(P.nthreads)
        for (int s = 0; s < ntau; s++) {
            for (int c = 0; c < nf; ++c) {
                R e = solar * cosf_(c, s) * shadowf(c, s);
                for (int k = P.dep_ptr[c]; k < P.dep_ptr[c + 1]; ++k) {
                    int g = P.dep_idx[k];
                    e = e + ((R)P.dep_vf[k] * solar * alb * cosf_(g, s) * shadowf(g, s));
                }
                illum[(size_t)c * ntau + s] = e;
            }
        }
    }

    // main.cpp:1351-1433 (Gauss-Seidel sweep in facet order, per step)
    void multiplescattering() {
        const R solar = (R)G.solar;
        const R alb = (R)P.albedo;
        const R acc = (R)P.scattering_accuracy;
#pragma omp parallel num_threads(P.nthreads)
        {
            std::vector<R> sp(nf), po(nf), pn(nf);
#pragma omp for schedule(dynamic)
            for (int s = 0; s < ntau; ++s) {
                for (int c = 0; c < nf; ++c) {
                    sp[c] = solar * cosf_(c, s) * shadowf(c, s);
                    po[c] = alb * illum[(size_t)c * ntau + s];
                }
                for (int it = 0; it < 100000; ++it) {
                    for (int c = 0; c < nf; ++c) {
                        const int d0 = P.dep_ptr[c], d1 = P.dep_ptr[c + 1];
                        if (d1 != d0) {
                            R before = R(0), after = R(0);
                            for (int k = d0; k < d1; ++k) {
                                int g = P.dep_idx[k];
                                if (g > c) after = after + ((R)P.dep_vf[k] * po[g]);
                                else before = before + ((R)P.dep_vf[k] * pn[g]);
                            }
                            pn[c] = alb * (sp[c] + after + before);
                        } else {
                            pn[c] = po[c];
                        }
                    }
                    int test = 0;
                    for (int c = 0; c < nf; ++c) {
                        if (std::fabs(pn[c] - po[c]) > acc) test = test + 1;
                        po[c] = pn[c];
                    }
                    if (test == 0) break;
                }
                for (int c = 0; c < nf; ++c) illum[(size_t)c * ntau + s] = pn[c] / alb;
            }
        }
    }

    // main.cpp:1439-1467
    void initialisetemperatures() {
        const R alb = (R)P.albedo;
        const R es = (R)P.eps * (R)SIGMA;
        for (int c = 0; c < nf; ++c) {
            R t = R(0);
            for (int s = 0; s != ntau; ++s) t = t + ((R(1) / ntau) * illum[(size_t)c * ntau + s]);
            t = Real<R>::pwq((R(1) - alb) * t / es);
            for (int i = 0; i != nx + 1; ++i) temp[(size_t)c * (nx + 1) + i] = t;
            for (int s = 0; s != ntau; ++s) { stemp0[(size_t)c * ntau + s] = t; stemp1[(size_t)c * ntau + s] = t; }
        }
    }

    // main.cpp:1473-1557
    void inertiadifference(R ti) {
        const R DZ = R(8) / nx;
        const R DTAU = R(2) * (R)(float)PI / ntau;
        const R alb = (R)P.albedo;
        const R E = (R)P.eps, S = (R)SIGMA;
        const R Pr = (R)P.rotation_period;
        const double tacc10 = (double)P.tacc / 10.0;
        std::vector<R> snap(nf);
        for (int s = 0; s != ntau; ++s) {
            for (int c = 0; c < nf; ++c) snap[c] = stemp1[(size_t)c * ntau + s];
#pragma omp parallel for schedule(static) num_threads(P.nthreads)
            for (int c = 0; c < nf; c++) {
                if (conv[c]) continue;
                R* T = &temp[(size_t)c * (nx + 1)];
                stemp0[(size_t)c * ntau + s] = stemp1[(size_t)c * ntau + s];
                R t0 = T[0];
                for (int i = 1; i != nx; ++i) {
                    R t1 = T[i];
                    T[i] = T[i] + ((DTAU / (DZ * DZ)) * (T[i + 1] - (R(2) * T[i]) + t0));
                    t0 = t1;
                }
                R inc = R(0);
                for (int k = P.dep_ptr[c]; k < P.dep_ptr[c + 1]; ++k)
                    inc = inc + (E * S * Real<R>::pw4(snap[P.dep_idx[k]]) * (R)P.dep_vf[k]);
                R DT = R(1);
                R TR0 = T[0], TR1 = T[0];
                int it = 0;
                while ((double)DT >= tacc10 && it < 10000) {
                    R SBC = ((R(1) - alb) * illum[(size_t)c * ntau + s]) + inc +
                            ((ti * std::sqrt(R(2) * (R)(float)PI / Pr) / DZ) * (T[1] - TR0)) -
                            (E * S * Real<R>::pw4(TR0));
                    R SBCD = (ti * std::sqrt(R(2) * (R)(float)PI / Pr) / DZ) + (R(4) * E * S * Real<R>::pw3(TR0));
                    TR1 = TR0 + (SBC / SBCD);
                    DT = std::fabs(TR1 - TR0);
                    TR0 = TR1;
                    ++it;
                }
                T[0] = TR1;
                stemp1[(size_t)c * ntau + s] = TR1;
                T[nx] = T[nx - 1];
            }
        }
    }

    // main.cpp:1563-1612
    void instequilibrium() {
        const R alb = (R)P.albedo;
        const R E = (R)P.eps, S = (R)SIGMA;
        std::vector<R> snap(nf);
        for (int s = 0; s != ntau; ++s) {
            for (int c = 0; c < nf; ++c) snap[c] = stemp1[(size_t)c * ntau + s];
            for (int c = 0; c < nf; c++) {
                stemp0[(size_t)c * ntau + s] = stemp1[(size_t)c * ntau + s];
                R inc = R(0);
                for (int k = P.dep_ptr[c]; k < P.dep_ptr[c + 1]; ++k)
                    inc = inc + (E * S * Real<R>::pw4(snap[P.dep_idx[k]]) * (R)P.dep_vf[k]);
                stemp1[(size_t)c * ntau + s] =
                    Real<R>::pwq((((R(1) - alb) * illum[(size_t)c * ntau + s]) + inc) / (E * S));
            }
        }
    }

    // main.cpp:1876-1909
    void shape_converged() {
        int all = 1;
        numconverged = 0;
        for (int c = 0; c < nf; ++c) {
            int fc = 1;
            for (int s = 0; s != ntau; ++s) {
                R DT = std::fabs(stemp1[(size_t)c * ntau + s] - stemp0[(size_t)c * ntau + s]);
                if (DT >= (R)P.tacc) { all = 0; fc = 0; }
            }
            if (fc == 1) { conv[c] = 1; numconverged = numconverged + 1; }
        }
        converged = all;
    }
};

template <class R>
void run(const oracle_params& P, const Geometry& G, oracle_outputs& O) {
    Thermal<R> T(P, G);
    T.singlescattering();
    if (P.multiple_scattering) T.multiplescattering();
    const size_t n = (size_t)P.nf * P.ntau;
    if (O.illumination)
        for (size_t i = 0; i < n; ++i) O.illumination[i] = (float)T.illum[i];
    if (O.illumination64)
        for (size_t i = 0; i < n; ++i) O.illumination64[i] = (double)T.illum[i];
    int initialised = 0;
    for (int k = 0; k < P.nti; ++k) {
        // reset_asteroid_status (main.cpp:477-485)
        T.numconverged = 0; T.converged = 0;
        std::fill(T.conv.begin(), T.conv.end(), 0);
        const float ti = P.ti[k];
        if (ti != 0.0f && !initialised) { T.initialisetemperatures(); initialised = 1; }
        int rev = 0;
        while (T.converged == 0 && rev < P.revcap) {
            if (ti == 0.0f) T.instequilibrium();
            else T.inertiadifference((R)ti);
            if (rev > 5) T.shape_converged();
            if (O.numconverged) O.numconverged[(size_t)k * P.revcap + rev] = T.numconverged;
            rev = rev + 1;
        }
        if (O.nrev) O.nrev[k] = rev;
    }
    for (size_t i = 0; i < n; ++i) {
        if (O.stemp1) O.stemp1[i] = (float)T.stemp1[i];
        if (O.stemp0) O.stemp0[i] = (float)T.stemp0[i];
        if (O.stemp1_64) O.stemp1_64[i] = (double)T.stemp1[i];
    }
    if (O.temp)
        for (size_t i = 0; i < (size_t)P.nf * (P.nx + 1); ++i) O.temp[i] = (float)T.temp[i];
}

}  // namespace

extern "C" {

// Geometry + shadowing only (main.cpp:894-1048, 1286-1315; Visibility 674-704).
int oracle_shadows(const oracle_params* P, int32_t* shadow, float* cosillum) {
    Geometry G;
    asteroidgeometry(*P, G);
    if (P->shadowing) {
#pragma omp parallel for schedule(dynamic) num_threads(P->nthreads)
        for (int s = 0; s < P->ntau; s++) {
            if (P->shadowing == 2) astshadow_allpairs(*P, G, s);
            else astshadow_deplist(*P, G, s);
        }
    }
    const size_t n = (size_t)P->nf * P->ntau;
    if (shadow) std::memcpy(shadow, G.shadow.data(), n * sizeof(int32_t));
    if (cosillum)
        for (size_t i = 0; i < n; ++i) cosillum[i] = (float)cos(G.illumangle[i]);
    return 0;
}

// Full single_model flow for a smooth shape (main.cpp:2417-2590, roughness off).
int oracle_single_model(const oracle_params* P, oracle_outputs* O) {
    Geometry G;
    asteroidgeometry(*P, G);
    if (P->shadowing) {
#pragma omp parallel for schedule(dynamic) num_threads(P->nthreads)
        for (int s = 0; s < P->ntau; s++) {
            if (P->shadowing == 2) astshadow_allpairs(*P, G, s);
            else astshadow_deplist(*P, G, s);
        }
    }
    const size_t n = (size_t)P->nf * P->ntau;
    if (O->shadow) std::memcpy(O->shadow, G.shadow.data(), n * sizeof(int32_t));
    if (O->cosillum)
        for (size_t i = 0; i < n; ++i) O->cosillum[i] = (float)cos(G.illumangle[i]);
    if (P->precision == 1) run<double>(*P, G, *O);
    else run<float>(*P, G, *O);
    return 0;
}

// glibc powf(x, e) over a float range, for pinning the device's pow tables.
void oracle_powf_range(const float* x, float e, float* out, int64_t n) {
    for (int64_t i = 0; i < n; ++i) out[i] = std::pow(x[i], e);
}

}  // extern "C"
