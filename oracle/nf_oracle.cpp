// nf_oracle.cpp -- CPU oracle of the NanoFiller hot path. TEST INFRASTRUCTURE:
// loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
//
// Build with -ffp-contract=off (oracle/Makefile): the FP64 decisions must be
// reproducible operation-for-operation, so no multiply-add may be fused.
//
// Reference lines restated here (pyrlinum/NanoFiller):
//   cnt_intersec_shr                inc/intersection_dev.h:10-80
//   distance_cylinder_capped        inc/intersect/intersect_cylinder_capped.h:69-147
//   if_intersects_cylinder_capped   inc/intersect/intersect_cylinder_capped.h:157-159
//   body_intersect_cylinder_capped  inc/intersect/intersect_cylinder_capped.h:181-183
//   surf_to_cylinder_capped         inc/intersect/intersect_cylinder_capped.h:204-293
//   generate_virt_inclusions        inc/conductKernels.h:289-361
//   stride2glbID_directed_uint      inc/memoryIO.h:70-85 (+ image shift stride2dspl :533-553)
//   set_numCNT                      src/simPrms.cpp:987-1002
//   get_elec_dmnID (electrode role) inc/conductivity.h:71-90 (plane form, see below)
//   kirchhoff assembly, G_eff       tools/kirchhoff/kirchhoff.py:232-269
#include "nf_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// ---------------------------------------------------------------------------
inline void philox(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t o[4]) {
    uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
    uint32_t k0 = k_in[0], k1 = k_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    o[0] = c0; o[1] = c1; o[2] = c2; o[3] = c3;
}

inline float uni(uint32_t u) { return (float)(u >> 8) * 5.9604644775390625e-08f; }

inline uint32_t fbits(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
inline float bitsf(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }

// sin/cos of 2*pi*t: quadrant reduction in turns (exact) + Taylor polynomials.
inline void sincos_turns(float t, float* c, float* s) {
    float t4 = t * 4.0f;
    float q = std::floor(t4 + 0.5f);
    float r = t4 - q;
    float x = r * (float)(M_PI / 2.0);
    float x2 = x * x;
    float ps = (float)(1.0 / 362880.0);
    ps = ps * x2 + (float)(-1.0 / 5040.0);
    ps = ps * x2 + (float)(1.0 / 120.0);
    ps = ps * x2 + (float)(-1.0 / 6.0);
    float sn = x + (x * x2) * ps;
    float pc = (float)(-1.0 / 3628800.0);
    pc = pc * x2 + (float)(1.0 / 40320.0);
    pc = pc * x2 + (float)(-1.0 / 720.0);
    pc = pc * x2 + (float)(1.0 / 24.0);
    pc = pc * x2 + -0.5f;
    float cs = 1.0f + x2 * pc;
    int qi = ((int)q) & 3;
    switch (qi) {
        case 0: *c = cs; *s = sn; break;
        case 1: *c = -sn; *s = cs; break;
        case 2: *c = -cs; *s = -sn; break;
        default: *c = sn; *s = -cs; break;
    }
}

// natural log via the atanh series of (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)).
inline float logf_nf(float v) {
    uint32_t b = fbits(v);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = bitsf((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421354f) { m = m * 0.5f; e += 1; }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = (float)(1.0 / 11.0);
    p = p * s2 + (float)(1.0 / 9.0);
    p = p * s2 + (float)(1.0 / 7.0);
    p = p * s2 + (float)(1.0 / 5.0);
    p = p * s2 + (float)(1.0 / 3.0);
    float two_s = s + s;
    float lm = two_s + two_s * (s2 * p);
    return (float)e * (float)M_LN2 + lm;
}

// exp via Cody-Waite reduction by ln2 and a degree-8 Taylor polynomial.
inline float expf_nf(float x) {
    float kf = std::floor(x * (float)(1.0 / M_LN2) + 0.5f);
    float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187e-06f;
    float p = (float)(1.0 / 40320.0);
    p = p * r + (float)(1.0 / 5040.0);
    p = p * r + (float)(1.0 / 720.0);
    p = p * r + (float)(1.0 / 120.0);
    p = p * r + (float)(1.0 / 24.0);
    p = p * r + (float)(1.0 / 6.0);
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    int k = (int)kf;
    if (k < -126) k = -126;
    if (k > 127) k = 127;
    return p * bitsf((uint32_t)(k + 127) << 23);
}

// ---------------------------------------------------------------------------
// FP64 erf / erfinv of the truncated-normal angle law (sym_truncNormal,
// inc/cuda_CNTgenerate.h:271-275), the product's operation sequence:
// ln by the atanh series to s^27, e^x by Cody-Waite + degree-13 Taylor, erf by
// its Maclaurin series below 2 and 1 - erfc (Laplace continued fraction, depth
// 50) above, erfinv by Winitzki's start (2008, a = 0.147) + two Halley steps.
// ---------------------------------------------------------------------------
inline uint64_t dbits(double v) { uint64_t u; std::memcpy(&u, &v, 8); return u; }
inline double bitsd(uint64_t u) { double v; std::memcpy(&v, &u, 8); return v; }
constexpr double kLn2Hi = 0.6931471803691238, kLn2Lo = 1.9082149292705877e-10;
constexpr double kInvLn2 = 1.4426950408889634, kSqrt2 = 1.4142135623730951;
constexpr double kSqrtPiHalf = 0.886226925452758, kTwoInvSqrtPi = 1.1283791670955126;
constexpr double kInvSqrtPi = 0.5641895835477563, kPiD = 3.141592653589793;
constexpr double kInv2PiD = 0.15915494309189535;

double log_d(double x) {
    const uint64_t b = dbits(x);
    int e = (int)((b >> 52) & 0x7ffu) - 1023;
    double m = bitsd((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
    if (m > kSqrt2) { m = m * 0.5; e += 1; }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double p = 1.0 / 27;
    for (int k = 25; k >= 3; k -= 2) p = p * s2 + 1.0 / k;
    const double two_s = s + s;
    const double lm = two_s + two_s * (s2 * p);
    return (double)e * kLn2Hi + ((double)e * kLn2Lo + lm);
}

double exp_d(double x) {
    static const double c[14] = {1.0, 1.0, 0.5, 0.16666666666666666, 0.041666666666666664, 0.008333333333333333,
                                 0.001388888888888889, 0.0001984126984126984, 2.48015873015873e-05,
                                 2.7557319223985893e-06, 2.755731922398589e-07, 2.505210838544172e-08,
                                 2.08767569878681e-09, 1.6059043836821613e-10};
    const double kf = std::floor(x * kInvLn2 + 0.5);
    const double r = (x - kf * kLn2Hi) - kf * kLn2Lo;
    double p = c[13];
    for (int n = 12; n >= 0; --n) p = p * r + c[n];
    int k = (int)kf;
    if (k < -1022) k = -1022;
    if (k > 1023) k = 1023;
    return p * bitsd((uint64_t)(k + 1023) << 52);
}

double erf_series(double x) {
    static const double c[35] = {1.0, 0.3333333333333333, 0.1, 0.023809523809523808, 0.004629629629629629,
                                 0.0007575757575757576, 0.00010683760683760684, 1.3227513227513228e-05,
                                 1.4589169000933706e-06, 1.4503852223150468e-07, 1.3122532963802806e-08,
                                 1.0892221037148573e-09, 8.35070279514724e-11, 5.9477940136376354e-12,
                                 3.9554295164585257e-13, 2.466827010264457e-14, 1.4483264643598138e-15,
                                 8.032735012415773e-17, 4.221407288807088e-18, 2.107855191442136e-19,
                                 1.0025164934907719e-20, 4.5518467589282e-22, 1.977064753877905e-23,
                                 8.230149299214221e-25, 3.289260349175752e-26, 1.2641078988989164e-27,
                                 4.6784835155184856e-29, 1.669761793417372e-30, 5.754191643982172e-32,
                                 1.9169428621097826e-33, 6.180307588222796e-35, 1.930357208815108e-36,
                                 5.846755007468836e-38, 1.7188560628017835e-39, 4.908923964523423e-41};
    const double mx2 = -(x * x);
    double p = c[34];
    for (int n = 33; n >= 0; --n) p = p * mx2 + c[n];
    return kTwoInvSqrtPi * (x * p);
}

double erfc_cf(double x) {
    double f = x;
    for (int k = 50; k >= 1; --k) f = x + ((double)k * 0.5) / f;
    return (exp_d(-(x * x)) * kInvSqrtPi) / f;
}

double erf_d(double x) {
    const double a = std::fabs(x);
    const double v = a < 2.0 ? erf_series(a) : 1.0 - erfc_cf(a);
    return x < 0.0 ? -v : v;
}

double erfinv_d(double y, double zmax) {
    const double a = std::fabs(y);
    double x;
    if (!(a < 1.0)) {
        x = zmax;
    } else {
        if (a < 1e-3) {
            x = kSqrtPiHalf * a;
        } else {
            const double L = log_d((1.0 - a) * (1.0 + a));
            const double A = 0.147;
            const double B = 2.0 / (kPiD * A) + L * 0.5;
            x = std::sqrt(std::sqrt(B * B - L / A) - B);
        }
        for (int it = 0; it < 2; ++it) {
            const double r = x < 2.0 ? erf_series(x) - a : (1.0 - a) - erfc_cf(x);
            const double d = (r * kSqrtPiHalf) * exp_d(x * x);
            x = x - d / (1.0 + x * d);
        }
        if (x > zmax) x = zmax;
    }
    return y < 0.0 ? -x : x;
}

// med + c2 erfinv(c1 (2u - 1)): one angle of the reference's law.
inline double tn_angle(float u, float med, double c1, double c2, double zmax) {
    const double v = c1 * (2.0 * (double)u - 1.0);
    return (double)med + c2 * erfinv_d(v, zmax);
}

// ---------------------------------------------------------------------------
// Derived stream constants (computed identically by the product's host code).
// ---------------------------------------------------------------------------
struct Stream {
    float L[3];
    uint32_t key[2];
    int orient, len_mode, rad_mode;
    float kappa, E2;
    bool rot;
    float m[9];
    // truncated-normal angle law: bit 0 theta, bit 1 phi
    int tn = 0;
    float tmed = 0, pmed = 0;
    double tc1 = 0, tc2 = 0, tz = 0, pc1 = 0, pc2 = 0, pz = 0;
    float l, a, sigma, lmin, lmax, rmin, rmax;
    // density
    const float* mesh;
    int n[3];
    float dflt;
    // per-cell orientation laws of the adaptive generation (null: the law above)
    const float* law = nullptr;
    const double* lawd = nullptr;  // ALIGN_LAW 1: kLawD doubles per cell
    int an[3] = {1, 1, 1};
    float ainv[3] = {0, 0, 0};
};

// Law layout: m[9] row-major (column 2 the axis), kappa, exp(-2 kappa),
// sampling flags (bit 0 von Mises-Fisher, bit 1 rotate, bit 2 the cell's own
// truncated-normal theta / phi laws), the cell's median theta and phi; the
// doubles: theta median and scale, phi median and scale, tn_angle's
// (c1, c2, zmax) for theta and for phi.
constexpr int kLawF = 14;
constexpr int kLawD = 10;

int law_cell(const Stream& S, float x, float y, float z) {
    const float v[3] = {x, y, z};
    int c[3];
    for (int d = 0; d < 3; ++d) {
        int i = (int)(v[d] * S.ainv[d]);
        c[d] = i < 0 ? 0 : (i >= S.an[d] ? S.an[d] - 1 : i);
    }
    return c[0] + S.an[0] * (c[1] + S.an[1] * c[2]);
}

// Constants of tn_angle for the scale s on +- w: the exact truncated normal,
// or the reference's own form (ref).
void tn_law(float sdev, double w, int ref, double* c1, double* c2, double* zmax) {
    const double sd = (double)sdev;
    const double z = (w / sd) / kSqrt2;
    if (ref) {
        *c1 = 0.5 * erf_d(z); *c2 = (2.0 * sd) * kSqrt2; *zmax = 1e300;
    } else {
        *c1 = erf_d(z); *c2 = sd * kSqrt2; *zmax = z;
    }
}

Stream make_stream(const nf_params* p, const float* mesh, int nx, int ny, int nz) {
    Stream S;
    for (int d = 0; d < 3; ++d) S.L[d] = p->box[d];
    S.key[0] = (uint32_t)(p->seed & 0xffffffffu);
    S.key[1] = (uint32_t)(p->seed >> 32);
    S.orient = p->orient_mode;
    S.len_mode = p->len_mode;
    S.rad_mode = p->rad_mode;
    S.kappa = p->vmf_kappa;
    S.E2 = (S.orient == NF_ORIENT_VMF) ? expf_nf(-2.0f * p->vmf_kappa) : 0.0f;
    S.rot = (p->pref_ort[0] != 0.0f) || (p->pref_ort[1] != 0.0f);
    float cM, sM, cX, sX;
    sincos_turns((float)((double)p->pref_ort[0] / (2.0 * M_PI)), &cM, &sM);
    sincos_turns((float)((double)(-p->pref_ort[1]) / (2.0 * M_PI)), &cX, &sX);
    // inc_rotation, inc/cuda_CNTgenerate.h:289-295 (Mu = phi, Xi = -theta)
    S.m[0] = cM * cX;  S.m[1] = sM;  S.m[2] = -sX * cM;
    S.m[3] = -sM * cX; S.m[4] = cM;  S.m[5] = sX * sM;
    S.m[6] = sX;       S.m[7] = 0.0f; S.m[8] = cX;
    // genCosine / sym_truncNormal (inc/cuda_CNTgenerate.h:262-275): theta
    // truncated to med +- pi/2, phi to med +- pi; exact normal by default,
    // the reference's 2 s sqrt2 erfinv(Fa (1 - 2u)) form on request (Q2)
    S.tn = (p->theta_dev > 0 ? 1 : 0) | (p->phi_dev > 0 ? 2 : 0);
    S.tmed = p->theta_med;
    S.pmed = p->phi_med;
    if (S.tn & 1) tn_law(p->theta_dev, kPiD * 0.5, p->ref_trunc_normal, &S.tc1, &S.tc2, &S.tz);
    if (S.tn & 2) tn_law(p->phi_dev, kPiD, p->ref_trunc_normal, &S.pc1, &S.pc2, &S.pz);
    S.l = p->l; S.a = p->a;
    S.sigma = p->len_sigma_ln; S.lmin = p->len_min; S.lmax = p->len_max;
    S.rmin = p->rad_min; S.rmax = p->rad_max;
    S.mesh = mesh;
    S.n[0] = nx; S.n[1] = ny; S.n[2] = nz;
    S.dflt = p->density_default;
    return S;
}

inline float lerpf(float a, float b, float f) { return a + (b - a) * f; }

float density(const Stream& S, float x, float y, float z) {
    if (!S.mesh) return S.dflt;
    float pos[3] = {x, y, z};
    int i0[3], i1[3];
    float f[3];
    for (int d = 0; d < 3; ++d) {
        float g = (pos[d] / S.L[d]) * (float)S.n[d] - 0.5f;
        float fl = std::floor(g);
        f[d] = g - fl;
        int i = (int)fl;
        i %= S.n[d];
        if (i < 0) i += S.n[d];
        i0[d] = i;
        i1[d] = (i + 1 == S.n[d]) ? 0 : i + 1;
    }
    auto v = [&](int i, int j, int k) { return S.mesh[((size_t)i * S.n[1] + j) * S.n[2] + k]; };
    float c00 = lerpf(v(i0[0], i0[1], i0[2]), v(i1[0], i0[1], i0[2]), f[0]);
    float c10 = lerpf(v(i0[0], i1[1], i0[2]), v(i1[0], i1[1], i0[2]), f[0]);
    float c01 = lerpf(v(i0[0], i0[1], i1[2]), v(i1[0], i0[1], i1[2]), f[0]);
    float c11 = lerpf(v(i0[0], i1[1], i1[2]), v(i1[0], i1[1], i1[2]), f[0]);
    float c0 = lerpf(c00, c10, f[1]);
    float c1 = lerpf(c01, c11, f[1]);
    return lerpf(c0, c1, f[2]);
}

// Candidate k: 10 floats x y z cx cy cz l a u rho.
void candidate(const Stream& S, uint64_t k, float* o) {
    uint32_t ctr[4] = {(uint32_t)k, (uint32_t)(k >> 32), 0u, 0u};
    uint32_t A[4], B[4];
    philox(ctr, S.key, A);
    ctr[2] = 1u;
    philox(ctr, S.key, B);
    float x = uni(A[0]) * S.L[0];
    float y = uni(A[1]) * S.L[1];
    float z = uni(A[2]) * S.L[2];
    float u = uni(A[3]);
    const float* m = S.m;
    float kappa = S.kappa, E2 = S.E2;
    bool vmf = S.orient == NF_ORIENT_VMF, rot = S.rot;
    float tmed = S.tmed, pmed = S.pmed;
    double tc1 = S.tc1, tc2 = S.tc2, tz = S.tz, pc1 = S.pc1, pc2 = S.pc2, pz = S.pz;
    if (S.law) {  // the law of the candidate's cell
        const int lc = law_cell(S, x, y, z);
        const float* Lw = S.law + (size_t)kLawF * lc;
        m = Lw;
        kappa = Lw[9];
        E2 = Lw[10];
        const int fl = (int)Lw[11];
        vmf = (fl & 1) != 0;
        rot = (fl & 2) != 0;
        if (fl & 4) {
            const double* Ld = S.lawd + (size_t)kLawD * lc;
            tmed = Lw[12];
            pmed = Lw[13];
            tc1 = Ld[4]; tc2 = Ld[5]; tz = Ld[6];
            pc1 = Ld[7]; pc2 = Ld[8]; pz = Ld[9];
        }
    }
    float cz;
    if (vmf) {
        float w = 1.0f - uni(B[0]);
        float v = w + (1.0f - w) * E2;
        cz = 1.0f + logf_nf(v) / kappa;
        if (cz < -1.0f) cz = -1.0f;
        if (cz > 1.0f) cz = 1.0f;
    } else if (S.tn & 1) {  // cos of a truncated-normal theta
        const double th = tn_angle(uni(B[0]), tmed, tc1, tc2, tz);
        float st;
        sincos_turns((float)(th * kInv2PiD), &cz, &st);
    } else {
        cz = uni(B[0]) * 2.0f - 1.0f;
    }
    float cp, sp;
    if (S.tn & 2) {  // truncated-normal phi
        const double ph = tn_angle(uni(B[1]), pmed, pc1, pc2, pz);
        sincos_turns((float)(ph * kInv2PiD), &cp, &sp);
    } else {
        sincos_turns(uni(B[1]), &cp, &sp);
    }
    float sr = 1.0f - cz * cz;
    float s = std::sqrt(sr > 0.0f ? sr : 0.0f);
    float cx = s * cp, cy = s * sp;
    if (rot) {
        float rx = (m[0] * cx + m[1] * cy) + m[2] * cz;
        float ry = (m[3] * cx + m[4] * cy) + m[5] * cz;
        float rz = (m[6] * cx + m[7] * cy) + m[8] * cz;
        cx = rx; cy = ry; cz = rz;
    }
    float len = S.l;
    if (S.len_mode == NF_SIZE_LOGNORMAL) {
        float cb, sb;
        sincos_turns(uni(B[3]), &cb, &sb);
        float g = std::sqrt(-2.0f * logf_nf(1.0f - uni(B[2]))) * cb;
        len = S.l * expf_nf(S.sigma * g);
        if (len < S.lmin) len = S.lmin;
        if (len > S.lmax) len = S.lmax;
    }
    float rad = S.a;
    if (S.rad_mode == NF_SIZE_UNIFORM) {
        uint32_t C[4];
        ctr[2] = 2u;
        philox(ctr, S.key, C);
        rad = S.rmin + (S.rmax - S.rmin) * uni(C[0]);
    }
    o[0] = x; o[1] = y; o[2] = z; o[3] = cx; o[4] = cy; o[5] = cz;
    o[6] = len; o[7] = rad; o[8] = u; o[9] = density(S, x, y, z);
}

// ---------------------------------------------------------------------------
// The reference routine, templated on the arithmetic type.
// A in "registers", B in "shared memory" shifted by its periodic image.
// ---------------------------------------------------------------------------
template <typename T>
struct RodT { T x, y, z, cx, cy, cz, l, a; };

template <typename T>
RodT<T> rodT(const nfo_rod& r) {
    return RodT<T>{(T)r.x, (T)r.y, (T)r.z, (T)r.cx, (T)r.cy, (T)r.cz, (T)r.l, (T)r.a};
}

template <typename T>
inline T tabs(T v) { return v < T(0) ? -v : v; }

// Returns d; writes clamped t0,t1 and Dtt (perpendicular distance, unclamped t0,t1).
template <typename T>
T ref_distance(const RodT<T>& A, const RodT<T>& B0, T sx, T sy, T sz, T eps, bool typo,
               T* t0o, T* t1o, T Dtt[3]) {
    const T Bx = B0.x + sx, By = B0.y + sy, Bz = B0.z + sz;  // tarnsCNT
    const T bx = Bx - A.x, by = By - A.y, bz = Bz - A.z;      // r2-r1
    T d = A.cx * B0.cx + A.cy * B0.cy + A.cz * B0.cz;           // c1*c2
    T t0, t1;
    if (T(1) - tabs(d) > eps) {
        T ax = d * B0.cx - A.cx, ay = d * B0.cy - A.cy, az = d * B0.cz - A.cz;
        t0 = ax * bx + ay * by + az * bz;
        ax = B0.cx - d * A.cx; ay = B0.cy - d * A.cy; az = B0.cz - d * A.cz;
        t1 = ax * bx + ay * by + az * bz;
        t0 = t0 / (d * d - T(1));
        t1 = t1 / (d * d - T(1));
    } else {
        t0 = std::copysign(A.l / T(2), bx * A.cx + by * A.cy + bz * A.cz);
        if (typo)
            t1 = T(-1) * (bx * B0.cx + bx * B0.cy + bx * B0.cz) + d * t0;
        else
            t1 = T(-1) * (bx * B0.cx + by * B0.cy + bz * B0.cz) + d * t0;
    }
    const T u0 = t0, u1 = t1;
    bool f1 = tabs(t0) <= (A.l / T(2) + A.a + eps);
    bool f2 = tabs(t1) <= (B0.l / T(2) + B0.a + eps);
    if (!(f1 && f2)) {
        bool f3 = (tabs(t0) - A.l / T(2)) < (tabs(t1) - B0.l / T(2));
        if (f3) {
            t1 = std::copysign(B0.l / T(2), t1);
            t0 = T(1) * (bx * A.cx + by * A.cy + bz * A.cz) + d * t1;
            T len = A.l / T(2);
            if (tabs(t0) > len) t0 = std::copysign(len, t0);
        } else {
            t0 = std::copysign(A.l / T(2), t0);
            t1 = T(-1) * (bx * B0.cx + by * B0.cy + bz * B0.cz) + d * t0;
            T len = B0.l / T(2);
            if (tabs(t1) > len) t1 = std::copysign(len, t1);
        }
    }
    T px = ((A.x + t0 * A.cx) - Bx) - t1 * B0.cx;
    T py = ((A.y + t0 * A.cy) - By) - t1 * B0.cy;
    T pz = ((A.z + t0 * A.cz) - Bz) - t1 * B0.cz;
    T dist = std::sqrt(px * px + py * py + pz * pz);
    T qx = ((A.x + u0 * A.cx) - Bx) - u1 * B0.cx;
    T qy = ((A.y + u0 * A.cy) - By) - u1 * B0.cy;
    T qz = ((A.z + u0 * A.cz) - Bz) - u1 * B0.cz;
    Dtt[0] = std::sqrt(qx * qx + qy * qy + qz * qz);
    Dtt[1] = u0;
    Dtt[2] = u1;
    *t0o = t0;
    *t1o = t1;
    return dist;
}

// threshold (a_B + a_A) * scf + sep + eps, left-to-right as in the reference.
template <typename T>
inline T thresh(T aA, T aB, T scf, T sep, T eps) { return (aB + aA) * scf + sep + eps; }

// ---------------------------------------------------------------------------
// Grid of cells with a 27-offset stencil and periodic images.
// ---------------------------------------------------------------------------
struct Grid {
    int n[3];
    float L[3];
    int periodic;
    double invE[3];
    void init(const float Lb[3], int per, double reach, double min_edge) {
        periodic = per;
        double e = std::max(reach * 1.0001, min_edge);
        for (int d = 0; d < 3; ++d) {
            L[d] = Lb[d];
            int c = (int)std::floor((double)Lb[d] / e);
            n[d] = c < 1 ? 1 : c;
            invE[d] = (double)n[d] / (double)Lb[d];
        }
    }
    int coord(int d, float x) const {
        int c = (int)std::floor((double)x * invE[d]);
        if (c < 0) c = 0;
        if (c >= n[d]) c = n[d] - 1;
        return c;
    }
    int ncell() const { return n[0] * n[1] * n[2]; }
};

struct Reach {  // per-run parameters of one pair kind
    double eps, scf, sep;
    int typo;
    int kind;
};

// d >= |b| - hA|cA| - hB|cB| (both points lie within h|c| of the centres), so
// pairs beyond this bound cannot satisfy the test; FP64 slack 1e-9 relative.
inline bool sphere_far(const RodT<double>& A, const RodT<double>& B, double sx, double sy,
                       double sz, double thr, double eps) {
    double bx = (B.x + sx) - A.x, by = (B.y + sy) - A.y, bz = (B.z + sz) - A.z;
    double nA = std::sqrt(A.cx * A.cx + A.cy * A.cy + A.cz * A.cz);
    double nB = std::sqrt(B.cx * B.cx + B.cy * B.cy + B.cz * B.cz);
    double R = ((A.l / 2 + A.a + eps) * nA + (B.l / 2 + B.a + eps) * nB + thr) * (1.0 + 1e-9) + 1e-12;
    return bx * bx + by * by + bz * bz > R * R;
}

// Hard-core test of candidate A against accepted B shifted by image.
inline bool hc_hit(const RodT<double>& A, const RodT<double>& B, double sx, double sy, double sz,
                   const nf_params* p, uint64_t* evals) {
    double eps = (double)p->tol, scf = (double)p->sc_frac, sep = (double)p->sep;
    if (!(A.l > 0)) return false;  // probe.l<=0
    double thr = thresh<double>(A.a, B.a, scf, sep, eps);
    if (sphere_far(A, B, sx, sy, sz, thr, eps)) return false;
    if (evals) ++*evals;
    double t0, t1, Dtt[3];
    double d = ref_distance<double>(A, B, sx, sy, sz, eps, p->ref_parallel_typo != 0, &t0, &t1, Dtt);
    return d < thr;
}

double gen_reach(const nf_params* p, double lmax, double amax) {
    double eps = p->tol;
    double h = lmax / 2 + amax + eps;
    return 2 * h + ((2 * amax) * p->sc_frac + p->sep + eps);
}

void size_bounds(const nf_params* p, double* lmax, double* amax) {
    *lmax = (p->len_mode == NF_SIZE_LOGNORMAL) ? (double)p->len_max : (double)p->l;
    *amax = (p->rad_mode == NF_SIZE_UNIFORM) ? (double)std::max(p->rad_min, p->rad_max) : (double)p->a;
}

int64_t target_count(const nf_params* p) {
    if (p->n_target > 0) return p->n_target;
    double V = (double)p->box[0] * p->box[1] * p->box[2];
    double El = p->l, Ea2 = (double)p->a * p->a;
    if (p->len_mode == NF_SIZE_LOGNORMAL) {
        // E[l] of the clipped lognormal by quadrature over the standard normal.
        double s = 0, w = 0;
        for (int i = -6000; i <= 6000; ++i) {
            double z = i * 1e-3, g = std::exp(-0.5 * z * z);
            double v = p->l * std::exp(p->len_sigma_ln * z);
            v = std::min(std::max(v, (double)p->len_min), (double)p->len_max);
            s += g * v; w += g;
        }
        El = s / w;
    }
    if (p->rad_mode == NF_SIZE_UNIFORM) {
        double lo = p->rad_min, hi = p->rad_max;
        Ea2 = (hi * hi + hi * lo + lo * lo) / 3.0;
    }
    double vinc = M_PI * Ea2 * El;
    return (int64_t)std::ceil((double)p->vf * V / vinc);
}

struct CellList {
    std::vector<std::vector<int64_t>> cells;
};

template <typename F>
void for_stencil(const Grid& g, const int c[3], F&& f) {
    for (int oz = -1; oz <= 1; ++oz)
        for (int oy = -1; oy <= 1; ++oy)
            for (int ox = -1; ox <= 1; ++ox) {
                int o[3] = {ox, oy, oz}, q[3], img[3];
                bool ok = true;
                for (int d = 0; d < 3; ++d) {
                    int v = c[d] + o[d];
                    img[d] = 0;
                    if (v < 0) {
                        if (!(g.periodic & (1 << d))) { ok = false; break; }
                        v += g.n[d]; img[d] = -1;
                    } else if (v >= g.n[d]) {
                        if (!(g.periodic & (1 << d))) { ok = false; break; }
                        v -= g.n[d]; img[d] = 1;
                    }
                    q[d] = v;
                }
                if (!ok) continue;
                int cell = q[0] + g.n[0] * (q[1] + g.n[1] * q[2]);
                f(cell, img);
            }
}

template <typename F>
void for_images(int periodic, F&& f) {
    for (int iz = -1; iz <= 1; ++iz)
        for (int iy = -1; iy <= 1; ++iy)
            for (int ix = -1; ix <= 1; ++ix) {
                int img[3] = {ix, iy, iz};
                bool ok = true;
                for (int d = 0; d < 3; ++d)
                    if (img[d] != 0 && !(periodic & (1 << d))) ok = false;
                if (ok) f(img);
            }
}

int nthreads_of(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// Union-find with path halving.
struct DSU {
    std::vector<int64_t> p;
    explicit DSU(int64_t n) : p(n) { std::iota(p.begin(), p.end(), 0); }
    int64_t find(int64_t x) {
        while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; }
        return x;
    }
    void unite(int64_t a, int64_t b) {
        a = find(a); b = find(b);
        if (a == b) return;
        if (a < b) std::swap(a, b);
        p[a] = b;
    }
};

// ---------------------------------------------------------------------------
// Adaptive generation (project-defined restatement of the reference's
// self-alignment, thin-out and clusterisation; src/cudaMain.cu:112-132,
// 254-273, 354-396, inc/allignment_fit.h, inc/cuda_Clusterize.h).
// ---------------------------------------------------------------------------
constexpr double kFix40 = 1099511627776.0;  // 2^40

void law_grid(const nf_params* p, int n[3], float inv[3]) {
    const double e = p->align_cell > 0 ? (double)p->align_cell : (double)p->l;
    for (int d = 0; d < 3; ++d) {
        const double c = std::floor((double)p->box[d] / e);
        n[d] = c < 1 ? 1 : (c > 256 ? 256 : (int)c);
        inv[d] = (float)((double)n[d] / (double)p->box[d]);
    }
}

// Eigen-decomposition of a symmetric 3x3 matrix by cyclic Jacobi rotations
// (Golub & Van Loan, Matrix Computations, sec. 8.5): A diagonal on return,
// eigenvectors in the columns of V.
void sym_eig3(double A[3][3], double V[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 64; ++sweep) {
        if (A[0][1] == 0.0 && A[0][2] == 0.0 && A[1][2] == 0.0) break;
        for (int r = 0; r < 3; ++r) {
            const int p = pairs[r][0], q = pairs[r][1];
            if (A[p][q] == 0.0) continue;
            const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
            const double at = th < 0 ? -th : th;
            double t = at > 1e150 ? 0.5 / at : 1.0 / (at + std::sqrt(th * th + 1.0));
            if (th < 0) t = -t;
            const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
            for (int k = 0; k < 3; ++k) {
                const double x = A[k][p], y = A[k][q];
                A[k][p] = c * x - sn * y;
                A[k][q] = sn * x + c * y;
            }
            for (int k = 0; k < 3; ++k) {
                const double x = A[p][k], y = A[q][k];
                A[p][k] = c * x - sn * y;
                A[q][k] = sn * x + c * y;
            }
            A[p][q] = A[q][p] = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double x = V[k][p], y = V[k][q];
                V[k][p] = c * x - sn * y;
                V[k][q] = sn * x + c * y;
            }
        }
    }
}

// E[(c.mu)^2] under a von Mises-Fisher law of concentration k.
double vmf_second_moment(double k) {
    if (k < 0.05) {
        const double k2 = k * k;
        return 1.0 / 3.0 + k2 * (2.0 / 45.0 - k2 * (4.0 / 945.0));
    }
    return 1.0 - 2.0 / (k * std::tanh(k)) + 2.0 / (k * k);
}

// A cell's law from its exact sums {n, xx, yy, zz, xy, xz, yz}.
void law_from_sums(const int64_t sm[7], bool sample, float* Lw) {
    const double f = 1.0 / ((double)sm[0] * kFix40);
    double A[3][3] = {{sm[1] * f, sm[4] * f, sm[5] * f}, {sm[4] * f, sm[2] * f, sm[6] * f},
                      {sm[5] * f, sm[6] * f, sm[3] * f}};
    double V[3][3];
    sym_eig3(A, V);
    int b = 0;
    for (int k = 1; k < 3; ++k)
        if (A[k][k] > A[b][b]) b = k;
    double mu[3] = {V[0][b], V[1][b], V[2][b]};
    const double nm = std::sqrt(mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]);
    for (int d = 0; d < 3; ++d) mu[d] /= nm;
    if (mu[2] < 0 || (mu[2] == 0 && (mu[1] < 0 || (mu[1] == 0 && mu[0] < 0))))
        for (int d = 0; d < 3; ++d) mu[d] = -mu[d];
    const double lam = A[b][b];
    double kap = 0.0;
    if (lam > 1.0 / 3.0 + 1e-9) {
        double lo = 0.0, hi = 500.0;
        if (vmf_second_moment(hi) <= lam) {
            kap = hi;
        } else {
            for (int it = 0; it < 64; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (vmf_second_moment(mid) < lam) lo = mid; else hi = mid;
            }
            kap = 0.5 * (lo + hi);
        }
    }
    // basis with mu as third column (Duff et al. 2017, "Building an
    // Orthonormal Basis, Revisited"); mu_z >= 0 here
    const double sg = mu[2] >= 0 ? 1.0 : -1.0;
    const double a = -1.0 / (sg + mu[2]), bb = mu[0] * mu[1] * a;
    const double e1[3] = {1.0 + sg * mu[0] * mu[0] * a, sg * bb, -sg * mu[0]};
    const double e2[3] = {bb, sg + mu[1] * mu[1] * a, -mu[1]};
    for (int r = 0; r < 3; ++r) {
        Lw[3 * r] = (float)e1[r];
        Lw[3 * r + 1] = (float)e2[r];
        Lw[3 * r + 2] = (float)mu[r];
    }
    const float kf = (float)kap;
    Lw[9] = kf;
    Lw[10] = (float)std::exp(-2.0 * (double)kf);
    Lw[11] = sample ? (float)((kf > 0.0f ? 1 : 0) | 2) : 0.0f;
}

// ALIGN_LAW 1: the reference's cell law (crossMtxBuild, resetOrt,
// resetAvgVec; inc/allignment_fit.h:154-210, 214-274, 353-458) from the
// directions of the cell's rods in rod order, in FP64: the preferred axis is
// the unit eigenvector of <c c^T> of the largest eigenvalue when the two
// smaller (by magnitude) are within 10 % of each other, else of the
// smallest, signed with v_z > 0; theta_o = acos(v_z), phi_o =
// acos(v_x / sin theta_o) (1e-6 guards), the draw rotated by
// inc_rotation(phi_o, -theta_o). When the unit-free mean direction has a norm
// per rod above 0.5 (def_minOrtNorm, src/simPrms.cpp:42), its box-frame
// angles (Ort2Angle, inc/vectorMath.h:85-90) are the medians and the mean
// squared deviations of the rods' angles from them the scales of the
// truncated-normal draws (the reference's rotation into the preferred frame
// discards its result, so the angles are box-frame angles).
void box_angles(double cx, double cy, double* th, double* ph) {
    const double nxy = std::sqrt(cx * cx + cy * cy);
    *th = std::asin(nxy > 1.0 ? 1.0 : nxy);
    double q = nxy > 1e-6 ? cx / nxy : 0.0;
    q = q > 1.0 ? 1.0 : (q < -1.0 ? -1.0 : q);
    *ph = nxy > 1e-6 ? std::acos(q) : 0.0;
}

void tn_cell_law(const std::vector<const nfo_rod*>& rs, int ref, float* Lw, double* Ld) {
    const double n = (double)rs.size();
    double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double ax = 0, ay = 0, az = 0;
    for (const nfo_rod* r : rs) {
        const double x = r->cx, y = r->cy, z = r->cz;
        A[0][0] += x * x; A[1][1] += y * y; A[2][2] += z * z;
        A[0][1] += x * y; A[0][2] += x * z; A[1][2] += y * z;
        ax += x; ay += y; az += z;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) A[i][j] /= n;
    A[1][0] = A[0][1]; A[2][0] = A[0][2]; A[2][1] = A[1][2];
    double V[3][3];
    sym_eig3(A, V);
    int o[3] = {0, 1, 2};
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (std::fabs(A[o[b]][o[b]]) > std::fabs(A[o[a]][o[a]])) std::swap(o[a], o[b]);
    const double e1 = A[o[1]][o[1]], e2 = A[o[2]][o[2]];
    const int k = std::fabs((e1 - e2) / e1) < 0.1 ? o[0] : o[2];
    double v[3] = {V[0][k], V[1][k], V[2][k]};
    const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int d = 0; d < 3; ++d) v[d] /= nv;
    if (v[2] < 0 || (v[2] == 0 && (v[1] < 0 || (v[1] == 0 && v[0] < 0))))
        for (int d = 0; d < 3; ++d) v[d] = -v[d];
    const double tho = std::fabs(v[2]) <= 1.0 - 1e-6 ? std::acos(v[2]) : (v[2] > 0 ? 0.0 : kPiD);
    const double sth = std::sin(tho);
    const double cph = std::fabs(sth) > 1e-6 ? v[0] / sth : 1.0;
    const double pho = std::fabs(cph) <= 1.0 - 1e-6 ? std::acos(cph) : (cph > 0 ? 0.0 : kPiD);
    float cM, sM, cX, sX;
    sincos_turns((float)(pho / (2.0 * kPiD)), &cM, &sM);
    sincos_turns((float)(-tho / (2.0 * kPiD)), &cX, &sX);
    Lw[0] = cM * cX;  Lw[1] = sM;   Lw[2] = -sX * cM;
    Lw[3] = -sM * cX; Lw[4] = cM;   Lw[5] = sX * sM;
    Lw[6] = sX;       Lw[7] = 0.0f; Lw[8] = cX;
    Lw[9] = 0.0f;
    Lw[10] = 0.0f;
    int fl = 2 | ((int)Lw[11] & 4);
    const double na = std::sqrt(ax * ax + ay * ay + az * az);
    if (na / n > 0.5) {
        double th, ph;
        box_angles(ax / na, ay / na, &th, &ph);
        double st = 0.0, sp = 0.0;
        for (const nfo_rod* r : rs) {
            double dt, dp;
            box_angles(r->cx, r->cy, &dt, &dp);
            st += (dt - th) * (dt - th);
            sp += (dp - ph) * (dp - ph);
        }
        const float ft = (float)th, fp = (float)ph;
        const float dt = std::max((float)(st / n), 1e-12f), dp = std::max((float)(sp / n), 1e-12f);
        Lw[12] = ft;
        Lw[13] = fp;
        Ld[0] = ft; Ld[1] = dt; Ld[2] = fp; Ld[3] = dp;
        tn_law(dt, kPiD * 0.5, ref, &Ld[4], &Ld[5], &Ld[6]);
        tn_law(dp, kPiD, ref, &Ld[7], &Ld[8], &Ld[9]);
        fl |= 4;
    }
    Lw[11] = (float)fl;
}

// Thin-out under ALIGN_LAW 1 (randomThinOut / check_probability,
// inc/allignment_fit.h:466-578): the rod stays when 2 F >= u, F the product of
// the Gaussian factors of its box-frame theta and phi under the cell's law.
bool tn_keep(const Stream& S, const float* Lw, const double* Ld, const nfo_rod& r, uint64_t si, uint32_t epoch) {
    if (!(((int)Lw[11]) & 4)) return true;
    double th, ph;
    box_angles(r.cx, r.cy, &th, &ph);
    const double qt = (th - Ld[0]) / Ld[1], qp = (ph - Ld[2]) / Ld[3];
    const double F = std::exp(-0.5 * qt * qt) * std::exp(-0.5 * qp * qp);
    uint32_t ctr[4] = {(uint32_t)si, (uint32_t)(si >> 32), 3u, epoch}, o[4];
    philox(ctr, S.key, o);
    return 2.0 * F >= (double)uni(o[0]);
}

inline float dotf(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

// cnt_minDist (inc/intersection_dev.h:85-160) in FP32; the parameters before
// the clamp in *t0u, *t1u.
float min_dist_f32(const float r1[3], const float c1[3], float l1, float a1, const float r2[3], const float c2[3],
                   float l2, float a2, float eps, bool typo, float* t0u, float* t1u) {
    const float b[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
    const float d = dotf(c1, c2);
    float t0, t1;
    if (1.0f - std::fabs(d) > eps) {
        float a[3] = {d * c2[0] - c1[0], d * c2[1] - c1[1], d * c2[2] - c1[2]};
        t0 = dotf(a, b);
        const float a2v[3] = {c2[0] - d * c1[0], c2[1] - d * c1[1], c2[2] - d * c1[2]};
        t1 = dotf(a2v, b);
        const float den = d * d - 1.0f;
        t0 /= den;
        t1 /= den;
    } else {
        t0 = std::copysign(l1 / 2.0f, dotf(b, c1));
        const float dt = typo ? (b[0] * c2[0] + b[0] * c2[1]) + b[0] * c2[2] : dotf(b, c2);
        t1 = -1.0f * dt + d * t0;
    }
    *t0u = t0;
    *t1u = t1;
    const float h1 = l1 / 2.0f, h2 = l2 / 2.0f;
    const bool f1 = std::fabs(t0) <= (h1 + a1) + eps;
    const bool f2 = std::fabs(t1) <= (h2 + a2) + eps;
    if (!(f1 && f2)) {
        if (std::fabs(t0) - h1 < std::fabs(t1) - h2) {
            t1 = std::copysign(h2, t1);
            t0 = dotf(b, c1) + d * t1;
            if (std::fabs(t0) > h1) t0 = std::copysign(h1, t0);
        } else {
            t0 = std::copysign(h1, t0);
            t1 = -1.0f * dotf(b, c2) + d * t0;
            if (std::fabs(t1) > h2) t1 = std::copysign(h2, t1);
        }
    }
    float e[3];
    for (int k = 0; k < 3; ++k) e[k] = ((r1[k] + t0 * c1[k]) - r2[k]) - t1 * c2[k];
    return std::sqrt(dotf(e, e));
}

// One clusterisation step (cuda_Clusterize2Old, inc/cuda_Clusterize.h:66-90):
// the candidate (r1, c1, l1, a1) against an older rod (r2, c2, l2, a2) already
// shifted to its image. Returns true when the candidate moved.
bool clu_snap(float r1[3], float c1[3], float l1, float a1, const float r2[3], const float c2[3], float l2,
              float a2, float eps, bool typo, float sep, float cos_lim, float dist_lim) {
    const float e[3] = {r1[0] - r2[0], r1[1] - r2[1], r1[2] - r2[2]};
    if (!(std::sqrt(dotf(e, e)) < std::max(l1, l2) * 0.5f)) return false;
    if (!(std::fabs(dotf(c1, c2)) >= cos_lim)) return false;
    float t0, t1;
    const float d = min_dist_f32(r1, c1, l1, a1, r2, c2, l2, a2, eps, typo, &t0, &t1);
    if (!(d <= dist_lim)) return false;
    const float qq[3] = {r2[0] + c2[0] * t1, r2[1] + c2[1] * t1, r2[2] + c2[2] * t1};
    float v[3];
    for (int k = 0; k < 3; ++k) v[k] = (r1[k] + c1[k] * t0) - qq[k];
    const float vc = dotf(v, c2);
    for (int k = 0; k < 3; ++k) v[k] = v[k] - c2[k] * vc;
    const float nv = std::sqrt(dotf(v, v));
    if (!(nv > 0.0f)) return false;  // the axes meet: no direction to move along
    const float inv = 1.0f / nv;
    for (int k = 0; k < 3; ++k) v[k] = v[k] * inv;
    const float sd = (a1 + a2) + sep;
    const float tt = dotf(c1, c2) * t0;
    for (int k = 0; k < 3; ++k) r1[k] = (qq[k] + v[k] * sd) - c2[k] * tt;
    for (int k = 0; k < 3; ++k) c1[k] = c2[k];
    return true;
}

}  // namespace

// ===========================================================================
extern "C" {

void nfo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    philox(ctr, key, out);
}
void nfo_sincos_turns(float t, float* c, float* s) { sincos_turns(t, c, s); }
double nfo_erf(double x) { return erf_d(x); }
double nfo_erfinv(double y, double zmax) { return erfinv_d(y, zmax); }
double nfo_log_d(double x) { return log_d(x); }
double nfo_exp_d(double x) { return exp_d(x); }
float nfo_logf(float v) { return logf_nf(v); }
float nfo_expf(float x) { return expf_nf(x); }

int nfo_pair_eval(int use_double, int kind, const nfo_rod* A, const nfo_rod* B,
                  const double shift[3], double eps, double scf, double thr_sep, int typo,
                  double out[6]) {
    if (use_double) {
        RodT<double> a = rodT<double>(*A), b = rodT<double>(*B);
        if (kind == 0 && !(a.l > 0)) { for (int i = 0; i < 6; ++i) out[i] = 0; return 0; }
        double t0, t1, Dtt[3];
        double d = ref_distance<double>(a, b, shift[0], shift[1], shift[2], eps,
                                        kind == 0 && typo, &t0, &t1, Dtt);
        out[0] = d; out[1] = t0; out[2] = t1; out[3] = Dtt[0]; out[4] = Dtt[1]; out[5] = Dtt[2];
        return d < thresh<double>(a.a, b.a, scf, thr_sep, eps);
    } else {
        RodT<float> a = rodT<float>(*A), b = rodT<float>(*B);
        if (kind == 0 && !(a.l > 0)) { for (int i = 0; i < 6; ++i) out[i] = 0; return 0; }
        float t0, t1, Dtt[3];
        float d = ref_distance<float>(a, b, (float)shift[0], (float)shift[1], (float)shift[2],
                                      (float)eps, kind == 0 && typo, &t0, &t1, Dtt);
        out[0] = d; out[1] = t0; out[2] = t1; out[3] = Dtt[0]; out[4] = Dtt[1]; out[5] = Dtt[2];
        return d < thresh<float>(a.a, b.a, (float)scf, (float)thr_sep, (float)eps);
    }
}

int nfo_screen_eval(const nfo_rod* A, const double vr[3], const double vc[3], double vl,
                    double va, const double shift[3], double eps) {
    RodT<double> a = rodT<double>(*A);
    RodT<double> v{vr[0], vr[1], vr[2], vc[0], vc[1], vc[2], vl, va};
    double t0, t1, Dtt[3];
    double d = ref_distance<double>(a, v, shift[0], shift[1], shift[2], eps, false, &t0, &t1, Dtt);
    // if_intersects (separation 0, soft_frac 1) and body_intersect on the virtual rod.
    bool hit = d < thresh<double>(a.a, v.a, 1.0, 0.0, eps);
    bool body = (v.l / 2.0 - tabs(Dtt[2])) > (v.a + eps);
    return hit && body;
}

double nfo_contact_area(const nfo_rod* A, const nfo_rod* B, const double shift[3],
                        double Dtt_x, double t1u, double t2u, double rlim) {
    // surf_to_cylinder_capped in FP64 (A = probe, B = shifted partner).
    const double PIv = 3.141593;  // PI of inc/vectorMath.h:7
    double l1 = A->l, l2 = B->l, a1 = A->a, a2 = B->a;
    double c1[3] = {A->cx, A->cy, A->cz}, c2[3] = {B->cx, B->cy, B->cz};
    double r1[3] = {A->x, A->y, A->z};
    double r2[3] = {B->x + shift[0], B->y + shift[1], B->z + shift[2]};
    auto dot = [](const double* u, const double* w) { return u[0] * w[0] + u[1] * w[1] + u[2] * w[2]; };
    double sg = std::copysign(1.0, dot(c1, c2));
    double c2p[3] = {c2[0] * sg, c2[1] * sg, c2[2] * sg};
    double dr1 = 0.0, dr2 = 0.0;
    double h1 = std::max(Dtt_x - a2 - rlim, 0.0);
    double h2 = std::max(Dtt_x - a1 - rlim, 0.0);
    if (h1 <= a1) dr1 = a1 * std::sqrt(1 - (h1 / a1) * (h1 / a1));
    if (h2 <= a2) dr2 = a2 * std::sqrt(1 - (h2 / a2) * (h2 / a2));
    double dr = std::min(dr1, dr2);
    double S = PIv * dr * dr;
    double t1 = t1u, t2 = t2u;
    double d = dot(c1, c2p);
    double sng = std::sqrt(std::max(1 - d * d, 0.0));
    if (tabs(t1) < (l1 / 2 - a1) && tabs(t2) < (l2 / 2 - a2)) {
        double ax1[3] = {c1[0] + c2p[0], c1[1] + c2p[1], c1[2] + c2p[2]};
        double n1 = std::sqrt(dot(ax1, ax1));
        for (int i = 0; i < 3; ++i) ax1[i] *= 1.0 / n1;
        double csg = std::sqrt(std::max(1 - sng * sng, 0.0));
        double sngh = std::sqrt((1 - csg) / 2.0);
        double t2p = std::copysign(t2, dot(c1, c2));
        double dt0p = (sngh > 1e-6 ? dr2 / sngh : l1 / 2);
        double dt0m = dt0p;
        double q[3];
        for (int i = 0; i < 3; ++i) q[i] = r1[i] + c1[i] * (l1 / 2 - t1);
        double dt1p = dot(q, ax1);
        for (int i = 0; i < 3; ++i) q[i] = r1[i] + c1[i] * (-l1 / 2 - t1);
        double dt1m = tabs(dot(q, ax1));
        for (int i = 0; i < 3; ++i) q[i] = r2[i] + c2p[i] * (l2 / 2 - t2p);
        double dt2p = dot(q, ax1);
        for (int i = 0; i < 3; ++i) q[i] = r2[i] + c2p[i] * (-l2 / 2 - t2p);
        double dt2m = tabs(dot(q, ax1));
        double Ap = std::max(dr, std::min(dt0p, std::min(dt1p, dt2p)));
        double Am = std::max(dr, std::min(dt0m, std::min(dt1m, dt2m)));
        S = std::max(S, 0.5 * PIv * dr * (Ap + Am));
    }
    if ((sng <= (std::max(a1, a2) / std::min(l1, l2))) && (tabs(t1) <= l1 / 2 + a1 || tabs(t2) <= l2 / 2 + a2)) {
        double b[3] = {r2[0] - r1[0], r2[1] - r1[1], r2[2] - r1[2]};
        double cb1 = dot(c1, b), cb2 = dot(c2, b);
        double t1a = std::copysign(l1 / 2, cb1), t1b = -1 * std::copysign(l1 / 2, cb1);
        double t2a = std::copysign(l2 / 2, cb2), t2b = -1 * std::copysign(l2 / 2, cb2);
        double q[3];
        for (int i = 0; i < 3; ++i) q[i] = r1[i] + c1[i] * t1a;
        double t1ac = dot(q, c1);
        for (int i = 0; i < 3; ++i) q[i] = r1[i] + c1[i] * t1b;
        double t1bc = dot(q, c1);
        for (int i = 0; i < 3; ++i) q[i] = b[i] + r1[i] + c2[i] * t2a;
        double t2ac = dot(q, c1);
        for (int i = 0; i < 3; ++i) q[i] = b[i] + r1[i] + c2[i] * t2b;
        double t2bc = dot(q, c1);
        double p1c = cb1 > 0 ? std::min(t1ac, t2ac) : std::max(t1ac, t2ac);
        double p2c = cb1 > 0 ? std::max(t1bc, t2bc) : std::min(t1bc, t2bc);
        S = std::max(S, tabs(p2c - p1c) * 2 * dr);
    }
    return S;
}

int64_t nfo_first_hits(const nf_params* p, const nfo_rod* probes, const uint64_t* k, int64_t m,
                       const nfo_rod* rods, const uint64_t* sidx, int64_t n, int nthreads, int64_t* out) {
    if (!p || (m && (!probes || !k || !out)) || (n && (!rods || !sidx))) return -1;
    const int nt = nthreads_of(nthreads);
    std::vector<RodT<double>> R(n);
    for (int64_t j = 0; j < n; ++j) R[j] = rodT<double>(rods[j]);
    const double L[3] = {(double)p->box[0], (double)p->box[1], (double)p->box[2]};
    #pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
    for (int64_t i = 0; i < m; ++i) {
        const RodT<double> A = rodT<double>(probes[i]);
        int64_t first = -1;
        for (int64_t j = 0; j < n && first < 0; ++j) {
            if (sidx[j] >= k[i]) continue;
            for_images(p->gen_periodic & 7, [&](const int img[3]) {
                if (first < 0 && hc_hit(A, R[j], img[0] * L[0], img[1] * L[1], img[2] * L[2], p, nullptr))
                    first = j;
            });
        }
        out[i] = first;
    }
    return m;
}

int nfo_clust_snap(const nf_params* p, const nfo_rod* cand, const nfo_rod* older, const float shift[3],
                   nfo_rod* out) {
    if (!p || !cand || !older || !out) return -1;
    float r1[3] = {cand->x, cand->y, cand->z}, c1[3] = {cand->cx, cand->cy, cand->cz};
    const float r2[3] = {older->x + shift[0], older->y + shift[1], older->z + shift[2]};
    const float c2[3] = {older->cx, older->cy, older->cz};
    const bool moved = clu_snap(r1, c1, cand->l, cand->a, r2, c2, older->l, older->a, p->tol,
                                p->ref_parallel_typo != 0, p->sep, (float)std::cos((double)p->clust_angl),
                                p->clust_dist);
    *out = nfo_rod{r1[0], r1[1], r1[2], c1[0], c1[1], c1[2], cand->l, cand->a};
    return moved ? 1 : 0;
}

int nfo_fit_law(const int64_t sums[7], int sample, float law[12]) {
    if (!sums || !law || sums[0] <= 0) return -1;
    law_from_sums(sums, sample != 0, law);
    return 0;
}

int nfo_tn_cell_law(const float* dirs, int64_t n, int ref, float law[14], double lawd[10]) {
    if (!dirs || !law || !lawd || n <= 0) return -1;
    std::vector<nfo_rod> rs((size_t)n);
    std::vector<const nfo_rod*> ptr((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        rs[i] = nfo_rod{0, 0, 0, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], 0, 0};
        ptr[i] = &rs[i];
    }
    for (int q = 0; q < kLawF; ++q) law[q] = 0.0f;
    for (int q = 0; q < kLawD; ++q) lawd[q] = 0.0;
    tn_cell_law(ptr, ref, law, lawd);
    return 0;
}

int nfo_candidates(const nf_params* p, const float* mesh, int nx, int ny, int nz, uint64_t k0,
                   uint64_t n, float* out) {
    if (!p || !out) return -1;
    Stream S = make_stream(p, mesh, nx, ny, nz);
    for (uint64_t i = 0; i < n; ++i) candidate(S, k0 + i, out + 10 * i);
    return 0;
}

int64_t nfo_generate(const nf_params* p, const float* mesh, int nx, int ny, int nz,
                     int nthreads, int64_t batch, int brute_force, int64_t cap, nfo_rod* rods,
                     uint64_t* stream_index, uint64_t stats[7], float* laws_out, int64_t laws_cap,
                     int32_t law_ext[3]) {
    if (!p || !rods) return -1;
    const int nt = nthreads_of(nthreads);
    Stream S = make_stream(p, mesh, nx, ny, nz);
    const int64_t target = target_count(p);
    double lmax, amax;
    size_bounds(p, &lmax, &amax);
    Grid g;
    g.init(p->box, p->gen_periodic, gen_reach(p, lmax, amax), p->cell_edge);
    std::vector<std::vector<int64_t>> cells(g.ncell());
    std::vector<RodT<double>> accD;
    accD.reserve((size_t)std::max<int64_t>(target, 0));
    std::vector<uint64_t> sidx_all;  // stream index of every accepted rod
    int64_t acc = 0;
    uint64_t k = 0, drawn = 0, dens_acc = 0, evals = 0;
    const uint64_t budget = p->n_candidates;
    if (batch < 1) batch = 1;
    std::vector<float> cand;
    std::vector<char> keep;
    std::vector<uint64_t> ev_thread(nt, 0);
    auto cell_of = [&](const RodT<double>& r, int c[3]) {
        c[0] = g.coord(0, (float)r.x); c[1] = g.coord(1, (float)r.y); c[2] = g.coord(2, (float)r.z);
    };
    // adaptive generation: epochs of epoch_len candidates, per-cell laws
    const bool adapt = p->self_align_step > 0 || p->clust_flag;
    const uint64_t epoch_len = adapt ? (p->epoch_candidates > 0 ? (uint64_t)p->epoch_candidates
                                                                : std::max<uint64_t>(1024, (uint64_t)target))
                                     : 0;
    std::vector<float> laws;
    std::vector<double> lawsd;
    int an[3] = {1, 1, 1};
    if (adapt) {
        float ainv[3];
        law_grid(p, an, ainv);
        const size_t nc = (size_t)an[0] * an[1] * an[2];
        laws.assign(nc * kLawF, 0.0f);
        for (size_t c = 0; c < nc; ++c) {  // every cell starts with the global law
            float* Lw = &laws[c * kLawF];
            for (int q = 0; q < 9; ++q) Lw[q] = S.m[q];
            Lw[9] = S.orient == NF_ORIENT_VMF ? S.kappa : 0.0f;
            Lw[10] = S.orient == NF_ORIENT_VMF ? S.E2 : 0.0f;
            Lw[11] = (float)((S.orient == NF_ORIENT_VMF ? 1 : 0) | (S.rot ? 2 : 0));
        }
        lawsd.assign(nc * kLawD, 0.0);
        S.law = laws.data();
        S.lawd = lawsd.data();
        for (int d = 0; d < 3; ++d) { S.an[d] = an[d]; S.ainv[d] = ainv[d]; }
    }
    uint64_t epochs = 0, refits = 0, thinned = 0, snapped = 0;
    uint64_t epoch_begun = ~0ull;
    int64_t epoch_count0 = 0, n_old = 0;
    const float cos_lim = (float)std::cos((double)p->clust_angl);
    const float Lf[3] = {p->box[0], p->box[1], p->box[2]};
    auto rebuild = [&]() {
        for (auto& c : cells) c.clear();
        if (brute_force) return;
        for (int64_t j = 0; j < acc; ++j) {
            int c[3];
            cell_of(accD[j], c);
            cells[c[0] + g.n[0] * (c[1] + g.n[1] * c[2])].push_back(j);
        }
    };
    // the refit after epoch e (and the thin-out that follows it)
    auto boundary = [&](uint64_t e, int64_t gained) {
        const int st = p->self_align_step;
        const bool refit = st > 0 && e > 0 &&
                           ((e % (uint64_t)st) == 0 || (double)gained < (double)(target - acc) / 100.0);
        if (!refit) return;
        const size_t nc = (size_t)an[0] * an[1] * an[2];
        if (p->align_law == 1) {  // the reference's truncated-normal cell laws
            std::vector<std::vector<const nfo_rod*>> members(nc);
            for (int64_t j = 0; j < acc; ++j) {
                const nfo_rod& r = rods[j];
                members[(size_t)law_cell(S, r.x, r.y, r.z)].push_back(&rods[j]);
            }
            const size_t need = p->align_min > 0 ? (size_t)p->align_min : 1;
            for (size_t c = 0; c < nc; ++c)
                if (members[c].size() >= need)
                    tn_cell_law(members[c], p->ref_trunc_normal, &laws[c * kLawF], &lawsd[c * kLawD]);
            ++refits;
            if (!p->reduce_flag) return;
            int64_t w = 0;
            for (int64_t j = 0; j < acc; ++j) {
                const nfo_rod& r = rods[j];
                const size_t c = (size_t)law_cell(S, r.x, r.y, r.z);
                if (!tn_keep(S, &laws[c * kLawF], &lawsd[c * kLawD], r, sidx_all[j], (uint32_t)(e + 1))) continue;
                rods[w] = rods[j];
                accD[w] = accD[j];
                sidx_all[w] = sidx_all[j];
                ++w;
            }
            thinned += (uint64_t)(acc - w);
            acc = w;
            accD.resize(acc);
            sidx_all.resize(acc);
            rebuild();
            return;
        }
        std::vector<int64_t> sums(7 * nc, 0);
        for (int64_t j = 0; j < acc; ++j) {
            const nfo_rod& r = rods[j];
            int64_t* sm = &sums[7 * (size_t)law_cell(S, r.x, r.y, r.z)];
            const double x = r.cx, y = r.cy, z = r.cz;
            const double pr[6] = {x * x, y * y, z * z, x * y, x * z, y * z};
            sm[0] += 1;
            for (int q = 0; q < 6; ++q) sm[1 + q] += (int64_t)std::llrint(pr[q] * kFix40);
        }
        const int64_t need = p->align_min > 0 ? p->align_min : 1;
        for (size_t c = 0; c < nc; ++c)
            if (sums[7 * c] >= need) law_from_sums(&sums[7 * c], p->orient_mode == NF_ORIENT_VMF, &laws[c * kLawF]);
        ++refits;
        if (!p->reduce_flag) return;
        // thin-out: keep when 2 exp(kappa (|c.mu| - 1)) >= u(stream index, 3, e + 1)
        int64_t w = 0;
        for (int64_t j = 0; j < acc; ++j) {
            const nfo_rod& r = rods[j];
            const float* Lw = &laws[(size_t)kLawF * law_cell(S, r.x, r.y, r.z)];
            bool kp = true;
            if (Lw[9] > 0.0f) {
                const float dd = std::fabs((r.cx * Lw[2] + r.cy * Lw[5]) + r.cz * Lw[8]);
                const float F = expf_nf(Lw[9] * (dd - 1.0f));
                const uint64_t si = sidx_all[j];
                uint32_t ctr[4] = {(uint32_t)si, (uint32_t)(si >> 32), 3u, (uint32_t)(e + 1)}, o[4];
                philox(ctr, S.key, o);
                kp = 2.0f * F >= uni(o[0]);
            }
            if (!kp) continue;
            rods[w] = rods[j];
            accD[w] = accD[j];
            sidx_all[w] = sidx_all[j];
            ++w;
        }
        thinned += (uint64_t)(acc - w);
        acc = w;
        accD.resize(acc);
        sidx_all.resize(acc);
        rebuild();
    };
    // clusterisation of one kept candidate o (x y z cx cy cz l a) onto the
    // rods [0, n_old); returns false when it leaves the box on an open axis
    auto clusterize = [&](float* o, uint64_t* nsnap) -> bool {
        const float h0[3] = {o[0], o[1], o[2]};
        std::vector<std::pair<int64_t, int>> nb;  // (rod, image code)
        auto visit = [&](int64_t j, const int img[3]) {
            if (j >= n_old) return;
            const nfo_rod& r = rods[j];
            float sh[3];
            for (int d = 0; d < 3; ++d) sh[d] = (float)img[d] * Lf[d];
            const float e[3] = {(r.x + sh[0]) - h0[0], (r.y + sh[1]) - h0[1], (r.z + sh[2]) - h0[2]};
            if (std::sqrt(dotf(e, e)) < std::max(o[6], r.l) * 0.5f)
                nb.push_back({j, (img[0] + 1) + 3 * (img[1] + 1) + 9 * (img[2] + 1)});
        };
        if (brute_force) {
            for (int64_t j = 0; j < n_old; ++j) for_images(g.periodic, [&](const int img[3]) { visit(j, img); });
        } else {
            RodT<double> A{};
            A.x = o[0]; A.y = o[1]; A.z = o[2];
            int c[3];
            cell_of(A, c);
            for_stencil(g, c, [&](int cell, const int img[3]) {
                for (int64_t j : cells[cell]) visit(j, img);
            });
        }
        std::sort(nb.begin(), nb.end());
        nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
        float r1[3] = {o[0], o[1], o[2]}, c1[3] = {o[3], o[4], o[5]};
        const float l1 = o[6], a1 = o[7];
        for (const auto& jb : nb) {
            const nfo_rod& q = rods[jb.first];
            const int im[3] = {jb.second % 3 - 1, (jb.second / 3) % 3 - 1, jb.second / 9 - 1};
            const float r2[3] = {q.x + (float)im[0] * Lf[0], q.y + (float)im[1] * Lf[1], q.z + (float)im[2] * Lf[2]};
            const float c2[3] = {q.cx, q.cy, q.cz};
            if (clu_snap(r1, c1, l1, a1, r2, c2, q.l, q.a, p->tol, p->ref_parallel_typo != 0, p->sep, cos_lim,
                         p->clust_dist))
                ++*nsnap;
        }
        bool inside = true;
        for (int d = 0; d < 3; ++d) {
            if (g.periodic & (1 << d)) {
                if (r1[d] < 0.0f) r1[d] = r1[d] + Lf[d];
                if (r1[d] >= Lf[d]) r1[d] = r1[d] - Lf[d];
            }
            if (!(r1[d] >= 0.0f && r1[d] < Lf[d])) inside = false;
        }
        for (int d = 0; d < 3; ++d) { o[d] = r1[d]; o[3 + d] = c1[d]; }
        return inside;
    };
    auto test_vs = [&](const RodT<double>& A, const std::vector<std::vector<int64_t>>& cl,
                       const std::vector<RodT<double>>& pool, uint64_t* ev) -> bool {
        if (brute_force) {
            bool hit = false;
            for (size_t j = 0; j < pool.size() && !hit; ++j)
                for_images(g.periodic, [&](const int img[3]) {
                    if (hit) return;
                    if (hc_hit(A, pool[j], img[0] * (double)g.L[0], img[1] * (double)g.L[1],
                               img[2] * (double)g.L[2], p, ev))
                        hit = true;
                });
            return hit;
        }
        int c[3];
        cell_of(A, c);
        bool hit = false;
        for_stencil(g, c, [&](int cell, const int img[3]) {
            if (hit) return;
            for (int64_t j : cl[cell]) {
                if (hc_hit(A, pool[j], img[0] * (double)g.L[0], img[1] * (double)g.L[1],
                           img[2] * (double)g.L[2], p, ev)) { hit = true; return; }
            }
        });
        return hit;
    };
    std::vector<uint32_t> snaps_c;  // snaps per candidate of the batch
    while (k < budget && acc < target) {
        if (adapt && k % epoch_len == 0 && k != epoch_begun) {
            if (k > 0) boundary(k / epoch_len - 1, acc - epoch_count0);
            epoch_begun = k;
            epoch_count0 = acc;
            n_old = acc;
            ++epochs;
            if (acc >= target) break;
        }
        uint64_t b = std::min<uint64_t>((uint64_t)batch, budget - k);
        if (adapt) b = std::min<uint64_t>(b, epoch_len - k % epoch_len);
        cand.assign(10 * b, 0.0f);
        keep.assign(b, 0);
        snaps_c.assign(b, 0);
        #pragma omp parallel for num_threads(nt) schedule(dynamic, 64)
        for (int64_t i = 0; i < (int64_t)b; ++i) {
            float* o = &cand[10 * i];
            candidate(S, k + i, o);
            if (!(o[8] < o[9])) continue;  // von Neumann: u < rho(x)
            keep[i] = 1;
#ifdef _OPENMP
            int tid = omp_get_thread_num();
#else
            int tid = 0;
#endif
            uint64_t ns = 0;
            const bool inside = !(adapt && p->clust_flag && n_old > 0) || clusterize(o, &ns);
            snaps_c[i] = (uint32_t)ns;
            if (!inside) {
                keep[i] = 2;  // moved out of the box
                continue;
            }
            nfo_rod r{o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]};
            RodT<double> A = rodT<double>(r);
            if (test_vs(A, cells, accD, &ev_thread[tid])) keep[i] = 2;  // hit an accepted rod
        }
        // In-batch conflicts, resolved in stream order.
        std::vector<std::vector<int64_t>> newcells(brute_force ? 0 : g.ncell());
        std::vector<RodT<double>> newD;
        uint64_t last = k + b;
        for (uint64_t i = 0; i < b; ++i) {
            if (keep[i] == 0) continue;
            ++dens_acc;
            if (keep[i] == 2) continue;
            float* o = &cand[10 * i];
            nfo_rod r{o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]};
            RodT<double> A = rodT<double>(r);
            if (test_vs(A, newcells, newD, &evals)) continue;
            if (acc >= cap) return -2;
            rods[acc] = r;
            accD.push_back(A);
            sidx_all.push_back(k + i);
            newD.push_back(A);
            if (!brute_force) {
                int c[3];
                cell_of(A, c);
                int cell = c[0] + g.n[0] * (c[1] + g.n[1] * c[2]);
                cells[cell].push_back((int64_t)accD.size() - 1);
                newcells[cell].push_back((int64_t)newD.size() - 1);
            }
            ++acc;
            if (acc == target) { last = k + i + 1; break; }
        }
        drawn = last;
        for (uint64_t i = 0; i < last - k; ++i) snapped += snaps_c[i];  // candidates consumed
        k += b;
    }
    if (acc < target) drawn = std::min<uint64_t>(k, budget);
    for (uint64_t e : ev_thread) evals += e;
    if (stream_index)
        for (int64_t j = 0; j < acc; ++j) stream_index[j] = sidx_all[j];
    if (stats) {
        stats[0] = drawn; stats[1] = dens_acc; stats[2] = evals;
        stats[3] = epochs; stats[4] = refits; stats[5] = thinned; stats[6] = snapped;
    }
    if (law_ext) for (int d = 0; d < 3; ++d) law_ext[d] = adapt ? an[d] : 0;
    if (laws_out && adapt && laws_cap >= (int64_t)laws.size())
        std::memcpy(laws_out, laws.data(), sizeof(float) * laws.size());
    return acc;
}

int64_t nfo_contacts(const nf_params* p, const nfo_rod* rods, int64_t n, int nthreads,
                     int brute_force, int64_t cap, uint32_t* I, uint32_t* J, double* tI,
                     double* tJ, double* D, double* G, double* S, int8_t* img, int64_t counts[4]) {
    if (!p || (!rods && n > 0)) return -1;
    const int nt = nthreads_of(nthreads);
    const double eps = 1e-6f;  // DEV_PRECISION, inc/definitions.h:5
    const double cut = p->stat_dist_lim;
    // peri_dir = 7 - dir; with buffer-layer electrodes the field axis is
    // periodic too: its images are the electrode layers
    const int fax = p->field_dir == 1 ? 0 : (p->field_dir == 2 ? 1 : (p->field_dir == 4 ? 2 : -1));
    const bool buf = p->elec_buffer && fax >= 0;
    const int per = buf ? ((p->gen_periodic | p->field_dir) & 7) : (p->gen_periodic & ~p->field_dir);
    double lmax = 0, amax = 0;
    for (int64_t i = 0; i < n; ++i) { lmax = std::max(lmax, (double)rods[i].l); amax = std::max(amax, (double)rods[i].a); }
    Grid g;
    double reach = 2 * (lmax / 2 + amax + eps) + (2 * amax + cut + eps);
    g.init(p->box, per, reach, p->cell_edge);
    std::vector<RodT<double>> R(n);
    std::vector<std::vector<int64_t>> cells(g.ncell());
    for (int64_t i = 0; i < n; ++i) {
        R[i] = rodT<double>(rods[i]);
        int c = g.coord(0, rods[i].x) + g.n[0] * (g.coord(1, rods[i].y) + g.n[1] * g.coord(2, rods[i].z));
        cells[c].push_back(i);
    }
    struct Ct { uint32_t i, j; int8_t im[3]; double t0, t1, d, Dx, u0, u1; };
    std::vector<std::vector<Ct>> per_t(nt);
    #pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
#ifdef _OPENMP
        auto& out = per_t[omp_get_thread_num()];
#else
        auto& out = per_t[0];
#endif
        const RodT<double>& A = R[i];
        auto test = [&](int64_t j, const int im[3]) {
            if (j <= i) return;
            const RodT<double>& B = R[j];
            double sx = im[0] * (double)g.L[0], sy = im[1] * (double)g.L[1], sz = im[2] * (double)g.L[2];
            double thr = thresh<double>(A.a, B.a, 1.0, cut, eps);
            if (sphere_far(A, B, sx, sy, sz, thr, eps)) return;
            double t0, t1, Dtt[3];
            double d = ref_distance<double>(A, B, sx, sy, sz, eps, false, &t0, &t1, Dtt);
            if (d < thr) {
                Ct c{(uint32_t)i, (uint32_t)j, {(int8_t)im[0], (int8_t)im[1], (int8_t)im[2]}, t0, t1, d, Dtt[0], Dtt[1], Dtt[2]};
                out.push_back(c);
            }
        };
        if (brute_force) {
            for (int64_t j = i + 1; j < n; ++j) for_images(per, [&](const int im[3]) { test(j, im); });
        } else {
            int c[3] = {g.coord(0, rods[i].x), g.coord(1, rods[i].y), g.coord(2, rods[i].z)};
            for_stencil(g, c, [&](int cell, const int im[3]) { for (int64_t j : cells[cell]) test(j, im); });
        }
    }
    std::vector<Ct> all;
    for (auto& v : per_t) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end(), [](const Ct& a, const Ct& b) {
        if (a.i != b.i) return a.i < b.i;
        if (a.j != b.j) return a.j < b.j;
        for (int d = 2; d >= 0; --d) if (a.im[d] != b.im[d]) return a.im[d] < b.im[d];
        return false;
    });
    // Screening by virtual inclusions (inc/conductKernels.h:289-361 and the
    // VIRTUAL_CHECK mode of src/core_cell_interaction_kernel.cu:141-146).
    std::vector<char> screened(all.size(), 0);
    if (p->screening) {
        double vreach = 2 * (lmax / 2 + amax + eps) + (2 * amax + eps);  // V shorter than a rod
        Grid gs;
        gs.init(p->box, per, vreach, p->cell_edge);
        std::vector<std::vector<int64_t>> rc(gs.ncell());
        for (int64_t i = 0; i < n; ++i)
            rc[gs.coord(0, rods[i].x) + gs.n[0] * (gs.coord(1, rods[i].y) + gs.n[1] * gs.coord(2, rods[i].z))].push_back(i);
        #pragma omp parallel for num_threads(nt) schedule(dynamic, 16)
        for (int64_t q = 0; q < (int64_t)all.size(); ++q) {
            const Ct& c = all[q];
            const RodT<double>& A = R[c.i];
            const RodT<double>& B = R[c.j];
            double sh[3] = {c.im[0] * (double)g.L[0], c.im[1] * (double)g.L[1], c.im[2] * (double)g.L[2]};
            double p0[3] = {A.x + c.t0 * A.cx, A.y + c.t0 * A.cy, A.z + c.t0 * A.cz};
            double p1[3] = {(B.x + sh[0]) + c.t1 * B.cx, (B.y + sh[1]) + c.t1 * B.cy, (B.z + sh[2]) + c.t1 * B.cz};
            double vr[3], vc[3];
            for (int d = 0; d < 3; ++d) { vr[d] = (p0[d] + p1[d]) * 0.5; vc[d] = p1[d] - p0[d]; }
            double vl = std::sqrt(vc[0] * vc[0] + vc[1] * vc[1] + vc[2] * vc[2]);
            if (!(vl > 0)) continue;
            for (int d = 0; d < 3; ++d) vc[d] = vc[d] * (1.0 / vl);
            double va = std::min(A.a, B.a);
            RodT<double> V{vr[0], vr[1], vr[2], vc[0], vc[1], vc[2], vl, va};
            // Cell of V's centre, wrapped into the box on periodic axes.
            int cc[3];
            double vw[3];
            for (int d = 0; d < 3; ++d) {
                double x = vr[d];
                if (per & (1 << d)) { x = std::fmod(x, (double)g.L[d]); if (x < 0) x += g.L[d]; }
                vw[d] = x;
                cc[d] = gs.coord(d, (float)x);
            }
            bool hit = false;
            for_stencil(gs, cc, [&](int cell, const int im[3]) {
                if (hit) return;
                for (int64_t r : rc[cell]) {
                    // real rod R[r] at image im relative to V's wrapped cell: the
                    // virtual rod is moved by -(image) so the real rod stays in place.
                    double sv[3];
                    for (int d = 0; d < 3; ++d) sv[d] = (vw[d] - vr[d]) - im[d] * (double)gs.L[d];
                    const RodT<double>& Rr = R[r];
                    double thr = thresh<double>(Rr.a, V.a, 1.0, 0.0, eps);
                    if (sphere_far(Rr, V, sv[0], sv[1], sv[2], thr, eps)) continue;
                    double t0, t1, Dtt[3];
                    double d = ref_distance<double>(Rr, V, sv[0], sv[1], sv[2], eps, false, &t0, &t1, Dtt);
                    if (d < thr && (V.l / 2.0 - tabs(Dtt[2])) > (V.a + eps)) { hit = true; return; }
                }
            });
            screened[q] = hit;
        }
    }
    // Buffer-layer electrodes (expand, src/simPrms.cpp:744-852, roles by
    // get_elec_dmnID, inc/conductivity.h:71-90): a kept pair whose partner is
    // an image across the field axis gives the rod whose partner lies below
    // the box a source contact and the other rod a sink contact.
    struct BufCt { uint32_t rod, partner; size_t q; bool iside; };
    std::vector<BufCt> bsnk, bsrc;
    std::vector<char> cross(all.size(), 0);
    if (buf)
        for (size_t q = 0; q < all.size(); ++q) {
            if (screened[q] || all[q].im[fax] == 0) continue;
            cross[q] = 1;
            const bool below = all[q].im[fax] < 0;
            bsrc.push_back({below ? all[q].i : all[q].j, below ? all[q].j : all[q].i, q, below});
            bsnk.push_back({below ? all[q].j : all[q].i, below ? all[q].i : all[q].j, q, !below});
        }
    auto bless = [](const BufCt& a, const BufCt& b) {
        if (a.rod != b.rod) return a.rod < b.rod;
        if (a.partner != b.partner) return a.partner < b.partner;
        return a.q < b.q;
    };
    std::sort(bsnk.begin(), bsnk.end(), bless);
    std::sort(bsrc.begin(), bsrc.end(), bless);
    int64_t n_int = 0, n_scr = 0;
    for (size_t q = 0; q < all.size(); ++q) if (!cross[q]) (screened[q] ? n_scr : n_int)++;
    // Electrode contacts: rods whose capsule comes within the cutoff of the
    // planes x_f = 0 (source) and x_f = L_f (sink) of the field axis f.
    std::vector<std::pair<uint32_t, double>> snk, src;  // (rod, D)
    std::vector<double> snk_t, src_t;
    int f = fax;
    if (f >= 0 && !buf) {
        for (int64_t i = 0; i < n; ++i) {
            const RodT<double>& A = R[i];
            double cf = f == 0 ? A.cx : (f == 1 ? A.cy : A.cz);
            double rf = f == 0 ? A.x : (f == 1 ? A.y : A.z);
            double half = A.l / 2;
            double tlo = cf > 0 ? -half : half;
            double thi = -tlo;
            double zlo = rf + tlo * cf, zhi = rf + thi * cf;
            double Lf = g.L[f];
            double dsnk = Lf - zhi;
            if (dsnk - A.a < cut + eps) { snk.push_back({(uint32_t)i, dsnk}); snk_t.push_back(thi); }
            if (zlo - A.a < cut + eps) { src.push_back({(uint32_t)i, zlo}); src_t.push_back(tlo); }
        }
    }
    const int64_t nsnk = (int64_t)(buf ? bsnk.size() : snk.size()), nsrc = (int64_t)(buf ? bsrc.size() : src.size());
    int64_t total = n_int + nsnk + nsrc;
    if (counts) { counts[0] = n_int; counts[1] = n_scr; counts[2] = nsnk; counts[3] = nsrc; }
    if (total > cap || !I) return total;
    const double G0 = p->G0, lam = p->lambda, dc = p->d_c;
    auto gfun = [&](double gap) { double ge = gap > dc ? gap : dc; return G0 * std::exp(-(ge - dc) / lam); };
    int64_t o = 0;
    for (size_t q = 0; q < all.size(); ++q) {
        if (screened[q] || cross[q]) continue;
        const Ct& c = all[q];
        I[o] = c.i; J[o] = c.j;
        if (tI) tI[o] = c.t0;
        if (tJ) tJ[o] = c.t1;
        if (D) D[o] = c.d;
        if (G) G[o] = gfun(c.d - R[c.i].a - R[c.j].a);
        if (S) {
            double sh[3] = {c.im[0] * (double)g.L[0], c.im[1] * (double)g.L[1], c.im[2] * (double)g.L[2]};
            S[o] = nfo_contact_area(&rods[c.i], &rods[c.j], sh, c.Dx, c.u0, c.u1, cut);
        }
        if (img) for (int d = 0; d < 3; ++d) img[3 * o + d] = c.im[d];
        ++o;
    }
    auto put_elec = [&](const std::vector<std::pair<uint32_t, double>>& v, const std::vector<double>& tv, uint32_t id) {
        for (size_t q = 0; q < v.size(); ++q) {
            I[o] = v[q].first; J[o] = id;
            if (tI) tI[o] = tv[q];
            if (tJ) tJ[o] = 0;
            if (D) D[o] = v[q].second;
            if (G) G[o] = gfun(v[q].second - R[v[q].first].a);
            if (S) S[o] = 0;
            if (img) for (int d = 0; d < 3; ++d) img[3 * o + d] = 0;
            ++o;
        }
    };
    auto put_buf = [&](const std::vector<BufCt>& v, uint32_t id) {
        for (const BufCt& b : v) {
            const Ct& c = all[b.q];
            I[o] = b.rod; J[o] = id;
            if (tI) tI[o] = b.iside ? c.t0 : c.t1;
            if (tJ) tJ[o] = b.iside ? c.t1 : c.t0;
            if (D) D[o] = c.d;
            if (G) G[o] = gfun(c.d - R[c.i].a - R[c.j].a);
            if (S) {
                double sh[3] = {c.im[0] * (double)g.L[0], c.im[1] * (double)g.L[1], c.im[2] * (double)g.L[2]};
                S[o] = nfo_contact_area(&rods[c.i], &rods[c.j], sh, c.Dx, c.u0, c.u1, cut);
            }
            if (img) for (int d = 0; d < 3; ++d) img[3 * o + d] = (int8_t)(b.iside ? c.im[d] : -c.im[d]);
            ++o;
        }
    };
    if (buf) {
        put_buf(bsnk, NF_SNK_ELEC);
        put_buf(bsrc, NF_SRC_ELEC);
    } else {
        put_elec(snk, snk_t, NF_SNK_ELEC);
        put_elec(src, src_t, NF_SRC_ELEC);
    }
    return total;
}

// Intra-rod resistor network (the `stat_conduct ... internal` mode):
// get_node_relations (src/conductivity.cu:639-754), get_internal_conduct and
// get_segment_length (:756-836, src/get_contact_data.cu:235-297),
// remove_redundant_nodes / reduce_node_tbl / recalculate_segments
// (src/adjacency_graph.cu:57-219), segment conductance s0 pi a / L
// (tools/kirchhoff/kirchhoff.py:90-95). Node positions t are the FP64 contact
// parameters; nodes are ordered by (rod, float(t)), ties in contact order.
static uint32_t ordered_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

int64_t nfo_internal_network(const nf_params* p, const nfo_rod* rods, int64_t n_rods, int64_t m,
                             const uint32_t* I, const uint32_t* J, const double* tI, const double* tJ,
                             int64_t cap, uint32_t* node_rod, double* node_t, uint32_t* seg_i, uint32_t* seg_j,
                             double* seg_l, double* seg_g, uint32_t* edge_i, uint32_t* edge_j, int64_t counts[3]) {
    if (!p || (m && (!I || !J || !tI || !tJ))) return -1;
    // slots 2e (rod I at tI) and 2e + 1 (rod J at tJ, internal contacts only)
    std::vector<std::pair<uint64_t, int64_t>> key;
    key.reserve(2 * m);
    for (int64_t e = 0; e < m; ++e) {
        key.push_back({((uint64_t)I[e] << 32) | ordered_bits((float)tI[e]), 2 * e});
        if (J[e] < NF_SNK_ELEC) key.push_back({((uint64_t)J[e] << 32) | ordered_bits((float)tJ[e]), 2 * e + 1});
    }
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<uint64_t, int64_t>& a, const std::pair<uint64_t, int64_t>& b) {
                         return a.first < b.first;
                     });
    const int64_t nfull = (int64_t)key.size();
    auto rod_of = [&](int64_t k) { return (uint32_t)(key[k].first >> 32); };
    auto t_of = [&](int64_t k) { int64_t sl = key[k].second; return (sl & 1) ? tJ[sl >> 1] : tI[sl >> 1]; };
    // A node merges into its predecessor on the same rod when the segment
    // between them is no longer than one radius (L = dt / a <= 1).
    std::vector<int64_t> group(nfull);
    int64_t ng = 0;
    for (int64_t k = 0; k < nfull; ++k) {
        bool merged = k > 0 && rod_of(k) == rod_of(k - 1) &&
                      (t_of(k) - t_of(k - 1)) / (double)rods[rod_of(k)].a <= 1.0;
        group[k] = merged ? ng - 1 : ng++;
    }
    if (ng > cap) return -2;
    std::vector<double> tsum(ng, 0.0);
    std::vector<int64_t> cnt(ng, 0);
    for (int64_t k = 0; k < nfull; ++k) { tsum[group[k]] += t_of(k); ++cnt[group[k]]; }
    for (int64_t k = 0; k < nfull; ++k) {
        node_rod[group[k]] = rod_of(k);
        node_t[group[k]] = tsum[group[k]] / (double)cnt[group[k]];
    }
    // contact ends -> nodes
    std::vector<uint32_t> node_of_slot(2 * m, 0xFFFFFFFFu);
    for (int64_t k = 0; k < nfull; ++k) node_of_slot[key[k].second] = (uint32_t)group[k];
    for (int64_t e = 0; e < m; ++e) {
        edge_i[e] = node_of_slot[2 * e];
        edge_j[e] = J[e] < NF_SNK_ELEC ? node_of_slot[2 * e + 1] : J[e];
    }
    // segments between consecutive nodes of a rod
    int64_t ns = 0;
    const double PIv = 3.14159265358979323846;
    for (int64_t g = 0; g + 1 < ng; ++g) {
        if (node_rod[g] != node_rod[g + 1]) continue;
        if (ns >= cap) return -2;
        const double a = (double)rods[node_rod[g]].a;
        const double L = (node_t[g + 1] - node_t[g]) / a;
        seg_i[ns] = (uint32_t)g;
        seg_j[ns] = (uint32_t)(g + 1);
        seg_l[ns] = L;
        seg_g[ns] = p->rod_sigma * PIv * a / L;
        ++ns;
    }
    (void)n_rods;
    counts[0] = ng;
    counts[1] = ns;
    counts[2] = nfull;
    return ng;
}

double nfo_solve(int64_t n_rods, int64_t n_contacts, const uint32_t* I, const uint32_t* J,
                 const double* G, double tol, int max_iter, double* v, double info[4]) {
    std::vector<double> s(n_rods, 0.0), t(n_rods, 0.0);
    DSU dsu(n_rods);
    for (int64_t e = 0; e < n_contacts; ++e) {
        if (J[e] == NF_SRC_ELEC) s[I[e]] += G[e];
        else if (J[e] == NF_SNK_ELEC) t[I[e]] += G[e];
        else dsu.unite(I[e], J[e]);
    }
    std::vector<char> hs(n_rods, 0), ht(n_rods, 0);
    for (int64_t i = 0; i < n_rods; ++i) {
        int64_t r = dsu.find(i);
        if (s[i] > 0) hs[r] = 1;
        if (t[i] > 0) ht[r] = 1;
    }
    std::vector<int64_t> idx(n_rods, -1);
    int64_t m = 0;
    for (int64_t i = 0; i < n_rods; ++i) {
        int64_t r = dsu.find(i);
        if (hs[r] && ht[r]) idx[i] = m++;
    }
    // Outside the source-sink network: components touching only the source sit
    // at 1 V, all others at 0 V (no current flows there either way).
    if (v) for (int64_t i = 0; i < n_rods; ++i) { int64_t r = dsu.find(i); v[i] = (hs[r] && !ht[r]) ? 1.0 : 0.0; }
    if (info) { info[0] = 0; info[1] = (double)m; info[2] = m > 0; info[3] = 0; }
    if (m == 0) return 0.0;
    // CSR of K = L + diag(s + t) on active nodes.
    std::vector<std::vector<std::pair<int64_t, double>>> rows(m);
    std::vector<double> diag(m, 0.0), b(m, 0.0);
    for (int64_t i = 0; i < n_rods; ++i) if (idx[i] >= 0) { diag[idx[i]] += s[i] + t[i]; b[idx[i]] = s[i]; }
    for (int64_t e = 0; e < n_contacts; ++e) {
        if (J[e] >= NF_SNK_ELEC) continue;
        int64_t a = idx[I[e]], c = idx[J[e]];
        if (a < 0) continue;
        diag[a] += G[e]; diag[c] += G[e];
        rows[a].push_back({c, -G[e]});
        rows[c].push_back({a, -G[e]});
    }
    auto spmv = [&](const std::vector<double>& x, std::vector<double>& y) {
        for (int64_t i = 0; i < m; ++i) {
            double acc = diag[i] * x[i];
            for (auto& kv : rows[i]) acc += kv.second * x[kv.first];
            y[i] = acc;
        }
    };
    std::vector<double> x(m, 0.0), r(b), z(m), pdir(m), q(m);
    double bn = std::sqrt(std::inner_product(b.begin(), b.end(), b.begin(), 0.0));
    for (int64_t i = 0; i < m; ++i) z[i] = r[i] / diag[i];
    pdir = z;
    double rz = std::inner_product(r.begin(), r.end(), z.begin(), 0.0);
    int it = 0;
    double rn = bn;
    for (; it < max_iter && rn > tol * bn; ++it) {
        spmv(pdir, q);
        double alpha = rz / std::inner_product(pdir.begin(), pdir.end(), q.begin(), 0.0);
        for (int64_t i = 0; i < m; ++i) { x[i] += alpha * pdir[i]; r[i] -= alpha * q[i]; }
        if ((it + 1) % 50 == 0) {  // true residual now and then
            spmv(x, q);
            for (int64_t i = 0; i < m; ++i) r[i] = b[i] - q[i];
        }
        rn = std::sqrt(std::inner_product(r.begin(), r.end(), r.begin(), 0.0));
        for (int64_t i = 0; i < m; ++i) z[i] = r[i] / diag[i];
        double rz2 = std::inner_product(r.begin(), r.end(), z.begin(), 0.0);
        double beta = rz2 / rz;
        rz = rz2;
        for (int64_t i = 0; i < m; ++i) pdir[i] = z[i] + beta * pdir[i];
    }
    spmv(x, q);
    double res = 0;
    for (int64_t i = 0; i < m; ++i) res += (b[i] - q[i]) * (b[i] - q[i]);
    double Geff = 0;
    for (int64_t i = 0; i < n_rods; ++i) {
        if (idx[i] < 0) continue;
        if (v) v[i] = x[idx[i]];
        Geff += s[i] * (1.0 - x[idx[i]]);
    }
    if (info) { info[0] = it; info[3] = std::sqrt(res) / bn; }
    return Geff;
}

void nfo_adjoint(const nf_params* p, const nfo_rod* rods, int64_t n_rods, int64_t n_contacts,
                 const uint32_t* I, const uint32_t* J, const double* tI, const double* tJ,
                 const double* D, const double* G, const int8_t* img, const double* v,
                 double* dG_dend, double* dG_dlambda, double* dG_dG0) {
    const double lam = p->lambda, dc = p->d_c, G0 = p->G0;
    double dl = 0, dg0 = 0;
    if (dG_dend) std::fill(dG_dend, dG_dend + 6 * n_rods, 0.0);
    int f = p->field_dir == 1 ? 0 : (p->field_dir == 2 ? 1 : (p->field_dir == 4 ? 2 : -1));
    for (int64_t e = 0; e < n_contacts; ++e) {
        uint32_t i = I[e], j = J[e];
        const nfo_rod& A = rods[i];
        double dv, gap;
        if (j == NF_SRC_ELEC) { dv = 1.0 - v[i]; gap = D[e] - A.a; }
        else if (j == NF_SNK_ELEC) { dv = v[i]; gap = D[e] - A.a; }
        else { dv = v[i] - v[j]; gap = D[e] - A.a - rods[j].a; }
        double w = dv * dv;  // dG_eff/dG_e (self-adjoint network)
        dg0 += w * G[e] / G0;
        bool clamped = !(gap > dc);
        if (!clamped) dl += w * G[e] * (gap - dc) / (lam * lam);
        if (!dG_dend || clamped) continue;
        double dGdD = -G[e] / lam * w;  // d/dD of G_e times dG_eff/dG_e
        if (j >= NF_SNK_ELEC) {
            // D = x_f of the lowest (source) / L - x_f of the highest (sink) axis end.
            double sgn = (j == NF_SRC_ELEC) ? 1.0 : -1.0;
            double uI = tI[e] / A.l + 0.5;
            dG_dend[6 * i + f] += dGdD * sgn * (1.0 - uI);
            dG_dend[6 * i + 3 + f] += dGdD * sgn * uI;
            continue;
        }
        const nfo_rod& B = rods[j];
        double sh[3] = {img[3 * e] * (double)p->box[0], img[3 * e + 1] * (double)p->box[1], img[3 * e + 2] * (double)p->box[2]};
        double pa[3] = {A.x + tI[e] * A.cx, A.y + tI[e] * A.cy, A.z + tI[e] * A.cz};
        double pb[3] = {(B.x + sh[0]) + tJ[e] * B.cx, (B.y + sh[1]) + tJ[e] * B.cy, (B.z + sh[2]) + tJ[e] * B.cz};
        double uI = tI[e] / A.l + 0.5, uJ = tJ[e] / B.l + 0.5;
        for (int d = 0; d < 3; ++d) {
            double gd = (pa[d] - pb[d]) / D[e] * dGdD;
            dG_dend[6 * i + d] += gd * (1.0 - uI);
            dG_dend[6 * i + 3 + d] += gd * uI;
            dG_dend[6 * j + d] -= gd * (1.0 - uJ);
            dG_dend[6 * j + 3 + d] -= gd * uJ;
        }
    }
    if (dG_dlambda) *dG_dlambda = dl;
    if (dG_dG0) *dG_dG0 = dg0;
}

}  // extern "C"
