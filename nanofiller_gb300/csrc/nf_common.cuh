// nf_common.cuh -- device-side building blocks shared by the GB300 kernels.
//
//  * no-contraction arithmetic: the seeded stream and the FP64 decision path
//    must give the same bits on the host (gcc, -ffp-contract=off) and on sm_103a,
//    so every multiply/add there goes through the _rn intrinsics;
//  * the project candidate stream (Philox4x32-10 + float transforms);
//  * the reference's pair routine in FP64 (cnt_intersec_shr,
//    inc/intersection_dev.h:10-80, and distance_cylinder_capped,
//    inc/intersect/intersect_cylinder_capped.h:69-147), one template body for
//    the hard-core and the contact test;
//  * the FP32 conservative filter that decides every far pair without FP64.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>
#include <cuda_runtime.h>

#define NF_HD __host__ __device__ __forceinline__

namespace nf {
// Kernel launches issued by this library (process-wide diagnostic).
extern unsigned long long g_launches;
// Device and pinned host blocks requested by this library, from cudaMalloc,
// cudaMallocHost or the block cache (process-wide diagnostic).
extern unsigned long long g_allocs;
}
#define NF_LAUNCH(kernel, ...) ++nf::g_launches, kernel<<<__VA_ARGS__>>>

namespace nf {

// ---------------------------------------------------------------------------
// Arithmetic without fused multiply-add.
// ---------------------------------------------------------------------------
#ifdef __CUDA_ARCH__
NF_HD float fmul(float a, float b) { return __fmul_rn(a, b); }
NF_HD float fadd(float a, float b) { return __fadd_rn(a, b); }
NF_HD float fsub(float a, float b) { return __fsub_rn(a, b); }
NF_HD float fdiv(float a, float b) { return __fdiv_rn(a, b); }
NF_HD float fsqrt(float a) { return __fsqrt_rn(a); }
NF_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
NF_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
NF_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
NF_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
NF_HD double dsqrt(double a) { return __dsqrt_rn(a); }
NF_HD uint32_t f2u(float f) { return __float_as_uint(f); }
NF_HD float u2f(uint32_t u) { return __uint_as_float(u); }
NF_HD uint32_t mulhi32(uint32_t a, uint32_t b) { return __umulhi(a, b); }
#else
NF_HD float fmul(float a, float b) { return a * b; }
NF_HD float fadd(float a, float b) { return a + b; }
NF_HD float fsub(float a, float b) { return a - b; }
NF_HD float fdiv(float a, float b) { return a / b; }
NF_HD float fsqrt(float a) { return sqrtf(a); }
NF_HD double dmul(double a, double b) { return a * b; }
NF_HD double dadd(double a, double b) { return a + b; }
NF_HD double dsub(double a, double b) { return a - b; }
NF_HD double ddiv(double a, double b) { return a / b; }
NF_HD double dsqrt(double a) { return sqrt(a); }
NF_HD uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
NF_HD float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
NF_HD uint32_t mulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((uint64_t)a * b) >> 32); }
#endif
NF_HD double dabs(double v) { return v < 0.0 ? -v : v; }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

NF_HD U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = mulhi32(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = mulhi32(0xCD9E8D57u, c2);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

NF_HD float uni(uint32_t u) { return fmul((float)(u >> 8), 5.9604644775390625e-08f); }

// sin/cos(2 pi t): exact quadrant reduction in turns, Taylor polynomials on
// [-pi/4, pi/4] (degree 9 / 10), Horner without fused multiply-add.
NF_HD void sincos_turns(float t, float* c, float* s) {
    float t4 = fmul(t, 4.0f);
    float q = floorf(fadd(t4, 0.5f));
    float r = fsub(t4, q);
    float x = fmul(r, (float)(3.14159265358979323846 / 2.0));
    float x2 = fmul(x, x);
    float ps = (float)(1.0 / 362880.0);
    ps = fadd(fmul(ps, x2), (float)(-1.0 / 5040.0));
    ps = fadd(fmul(ps, x2), (float)(1.0 / 120.0));
    ps = fadd(fmul(ps, x2), (float)(-1.0 / 6.0));
    float sn = fadd(x, fmul(fmul(x, x2), ps));
    float pc = (float)(-1.0 / 3628800.0);
    pc = fadd(fmul(pc, x2), (float)(1.0 / 40320.0));
    pc = fadd(fmul(pc, x2), (float)(-1.0 / 720.0));
    pc = fadd(fmul(pc, x2), (float)(1.0 / 24.0));
    pc = fadd(fmul(pc, x2), -0.5f);
    float cs = fadd(1.0f, fmul(x2, pc));
    int qi = ((int)q) & 3;
    if (qi == 0) { *c = cs; *s = sn; }
    else if (qi == 1) { *c = -sn; *s = cs; }
    else if (qi == 2) { *c = -cs; *s = -sn; }
    else { *c = sn; *s = -cs; }
}

// ln v (v > 0, normal): exponent split, mantissa in [sqrt(1/2), sqrt(2)),
// ln m = 2 atanh((m-1)/(m+1)) by its odd series to s^11.
NF_HD float log_nf(float v) {
    uint32_t b = f2u(v);
    int e = (int)((b >> 23) & 0xffu) - 127;
    float m = u2f((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421354f) { m = fmul(m, 0.5f); e += 1; }
    float s = fdiv(fsub(m, 1.0f), fadd(m, 1.0f));
    float s2 = fmul(s, s);
    float p = (float)(1.0 / 11.0);
    p = fadd(fmul(p, s2), (float)(1.0 / 9.0));
    p = fadd(fmul(p, s2), (float)(1.0 / 7.0));
    p = fadd(fmul(p, s2), (float)(1.0 / 5.0));
    p = fadd(fmul(p, s2), (float)(1.0 / 3.0));
    float two_s = fadd(s, s);
    float lm = fadd(two_s, fmul(two_s, fmul(s2, p)));
    return fadd(fmul((float)e, (float)0.69314718055994530942), lm);
}

// e^x: Cody-Waite reduction by ln 2, degree-8 Taylor polynomial, 2^k scaling.
NF_HD float exp_nf(float x) {
    float kf = floorf(fadd(fmul(x, (float)(1.0 / 0.69314718055994530942)), 0.5f));
    float r = fsub(fsub(x, fmul(kf, 0.693145751953125f)), fmul(kf, 1.428606765330187e-06f));
    float p = (float)(1.0 / 40320.0);
    p = fadd(fmul(p, r), (float)(1.0 / 5040.0));
    p = fadd(fmul(p, r), (float)(1.0 / 720.0));
    p = fadd(fmul(p, r), (float)(1.0 / 120.0));
    p = fadd(fmul(p, r), (float)(1.0 / 24.0));
    p = fadd(fmul(p, r), (float)(1.0 / 6.0));
    p = fadd(fmul(p, r), 0.5f);
    p = fadd(fmul(p, r), 1.0f);
    p = fadd(fmul(p, r), 1.0f);
    int k = (int)kf;
    k = k < -126 ? -126 : (k > 127 ? 127 : k);
    return fmul(p, u2f((uint32_t)(k + 127) << 23));
}

// ---------------------------------------------------------------------------
// FP64 error function and its inverse, for the truncated-normal angle law
// (sym_truncNormal, inc/cuda_CNTgenerate.h:271-275). Written from the
// mathematics, one operation sequence on host and device (no fused
// multiply-add), so the oracle reproduces every bit:
//  * ln x: exponent split, 2 atanh((m-1)/(m+1)) by its odd series to s^27;
//  * e^x: Cody-Waite reduction by ln 2 (high part with 32 significant bits),
//    Taylor polynomial of degree 13, 2^k scaling;
//  * erf x: Maclaurin series (35 terms, Horner in -x^2) below 2; above,
//    1 - erfc x with erfc from the Laplace continued fraction
//    e^{-x^2} / (sqrt(pi) (x + (1/2)/(x + 1/(x + (3/2)/(x + ...))))),
//    evaluated bottom-up to depth 50;
//  * erfinv y: the closed-form start of Winitzki ("A handy approximation for
//    the error function and its inverse", 2008; a = 0.147), or sqrt(pi)/2 y
//    below 1e-3, then two Halley steps on erf (residual formed from erfc
//    above 2, where 1 - |y| is exact).
// Relative error against 50-digit arithmetic: ln and e^x below 3e-16, erf below
// 1e-15, erfinv below 2e-14 down to 1 - |y| = 1e-16.
// ---------------------------------------------------------------------------
#ifdef __CUDA_ARCH__
NF_HD uint64_t d2u(double v) { return (uint64_t)__double_as_longlong(v); }
NF_HD double u2d(uint64_t u) { return __longlong_as_double((long long)u); }
#else
NF_HD uint64_t d2u(double v) { uint64_t u; memcpy(&u, &v, 8); return u; }
NF_HD double u2d(uint64_t u) { double v; memcpy(&v, &u, 8); return v; }
#endif
constexpr double kLn2Hi = 0.6931471803691238;      // ln 2 rounded to 32 bits
constexpr double kLn2Lo = 1.9082149292705877e-10;  // ln 2 - kLn2Hi
constexpr double kInvLn2 = 1.4426950408889634;
constexpr double kSqrt2 = 1.4142135623730951;
constexpr double kSqrtPiHalf = 0.886226925452758;  // sqrt(pi) / 2
constexpr double kTwoInvSqrtPi = 1.1283791670955126;
constexpr double kInvSqrtPi = 0.5641895835477563;
constexpr double kPiD = 3.141592653589793;
constexpr double kInv2PiD = 0.15915494309189535;
constexpr double kErfSplit = 2.0;

NF_HD double log_d(double x) {
    const uint64_t b = d2u(x);
    int e = (int)((b >> 52) & 0x7ffu) - 1023;
    double m = u2d((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
    if (m > kSqrt2) { m = dmul(m, 0.5); e += 1; }
    const double s = ddiv(dsub(m, 1.0), dadd(m, 1.0));
    const double s2 = dmul(s, s);
    double p = 1.0 / 27;
#pragma unroll
    for (int k = 25; k >= 3; k -= 2) p = dadd(dmul(p, s2), 1.0 / k);
    const double two_s = dadd(s, s);
    const double lm = dadd(two_s, dmul(two_s, dmul(s2, p)));
    return dadd(dmul((double)e, kLn2Hi), dadd(dmul((double)e, kLn2Lo), lm));
}

NF_HD double exp_d(double x) {
    const double c[14] = {1.0, 1.0, 0.5, 0.16666666666666666, 0.041666666666666664, 0.008333333333333333,
                          0.001388888888888889, 0.0001984126984126984, 2.48015873015873e-05,
                          2.7557319223985893e-06, 2.755731922398589e-07, 2.505210838544172e-08,
                          2.08767569878681e-09, 1.6059043836821613e-10};
    const double kf = floor(dadd(dmul(x, kInvLn2), 0.5));
    const double r = dsub(dsub(x, dmul(kf, kLn2Hi)), dmul(kf, kLn2Lo));
    double p = c[13];
#pragma unroll
    for (int n = 12; n >= 0; --n) p = dadd(dmul(p, r), c[n]);
    int k = (int)kf;
    k = k < -1022 ? -1022 : (k > 1023 ? 1023 : k);
    return dmul(p, u2d((uint64_t)(k + 1023) << 52));
}

// erf x for 0 <= x < 2: 2/sqrt(pi) sum_n (-1)^n x^(2n+1) / (n! (2n+1)).
NF_HD double erf_series(double x) {
    const double c[35] = {1.0, 0.3333333333333333, 0.1, 0.023809523809523808, 0.004629629629629629,
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
    const double mx2 = -dmul(x, x);
    double p = c[34];
#pragma unroll
    for (int n = 33; n >= 0; --n) p = dadd(dmul(p, mx2), c[n]);
    return dmul(kTwoInvSqrtPi, dmul(x, p));
}

// erfc x for x >= 2: the Laplace continued fraction, depth 50.
NF_HD double erfc_cf(double x) {
    double f = x;
    for (int k = 50; k >= 1; --k) f = dadd(x, ddiv(dmul((double)k, 0.5), f));
    return ddiv(dmul(exp_d(-dmul(x, x)), kInvSqrtPi), f);
}

NF_HD double erf_d(double x) {
    const double a = dabs(x);
    const double v = a < kErfSplit ? erf_series(a) : dsub(1.0, erfc_cf(a));
    return x < 0.0 ? -v : v;
}

// erfinv y, its magnitude capped at zmax (|y| >= 1 gives +-zmax).
NF_HD double erfinv_d(double y, double zmax) {
    const double a = dabs(y);
    double x;
    if (!(a < 1.0)) {
        x = zmax;
    } else {
        if (a < 1e-3) {
            x = dmul(kSqrtPiHalf, a);
        } else {
            const double L = log_d(dmul(dsub(1.0, a), dadd(1.0, a)));
            const double A = 0.147;
            const double B = dadd(ddiv(2.0, dmul(kPiD, A)), dmul(L, 0.5));
            x = dsqrt(dsub(dsqrt(dsub(dmul(B, B), ddiv(L, A))), B));
        }
        for (int it = 0; it < 2; ++it) {
            const double r = x < kErfSplit ? dsub(erf_series(x), a) : dsub(dsub(1.0, a), erfc_cf(x));
            const double d = dmul(dmul(r, kSqrtPiHalf), exp_d(dmul(x, x)));
            x = dsub(x, ddiv(d, dadd(1.0, dmul(x, d))));
        }
        if (x > zmax) x = zmax;
    }
    return y < 0.0 ? -x : x;
}

// One angle of the reference's law: med + c2 erfinv(c1 (2u - 1)), where
// (c1, c2, zmax) = (erf z, s sqrt 2, z) with z = w / (s sqrt 2) for the exact
// normal of deviation s truncated to med +- w, or (erf(z) / 2, 2 s sqrt 2,
// inf) for the reference's own form a + 2 s sqrt2 erfinv(Fa (1 - 2u)),
// Fa = erf(-z) / 2 (Fa (1 - 2u) = (erf(z) / 2)(2u - 1): erf is odd).
NF_HD double tn_angle(float u, float med, double c1, double c2, double zmax) {
    const double v = dmul(c1, dsub(dmul(2.0, (double)u), 1.0));
    return dadd((double)med, dmul(c2, erfinv_d(v, zmax)));
}

// ---------------------------------------------------------------------------
// Realisation descriptor: stream, density, grid, thresholds.
// ---------------------------------------------------------------------------
struct Real {
    // stream
    float L[3];
    uint32_t key[2];
    int32_t orient, len_mode, rad_mode, rot;
    float kappa, E2;
    float m[9];
    // the reference's truncated-normal angle law (DEF_THETA_*/DEF_PHI_*):
    // bit 0 theta, bit 1 phi drawn by tn_angle with (c1, c2, zmax)
    int32_t tn;
    float tmed, pmed;
    double tc1, tc2, tz, pc1, pc2, pz;
    float l, a, sigma, lmin, lmax, rmin, rmax;
    // density
    const float* mesh;
    int32_t mn[3];
    float dflt;
    // cell grid (shared by generation, contacts and screening); every pair
    // within reach is at most S cells apart along each axis
    int32_t n[3];
    float invE[3];
    int32_t S;
    int32_t per_gen, per_con;
    uint32_t cell_off, ncell;
    // tube grid of the pair sweeps (tube == 0: the cell-stencil sweeps): tcn
    // cells of edge tce = L / tcn across the box per axis (tci = 1 / tce), tcm
    // margin cells beyond each
    // face of an axis open in some stage; every object registers in each cell
    // that its axis segment, extended to l/2 + a + eps and dilated by trho,
    // touches (tube_walk)
    int32_t tube;
    int32_t tcn[3], tcm[3];
    float tci[3], tce[3];
    float trho;
    uint32_t toff, tncell;
    // rods
    uint32_t rod_off, target;
    // hard core (cnt_intersec_shr) and contacts (distance_cylinder_capped)
    float eps, scf, sep, cut;
    int32_t typo;
    float slack;            // FP32 filter: absolute slack for coordinate rounding
    int32_t field_axis;     // 0,1,2 or -1
    int32_t ebuf;           // electrodes are buffer layers of images (else planes)
    double G0, lambda, dc;
    // per-cell orientation laws of the adaptive generation (null: the global
    // law above): kLawF floats per law cell, grid an[] with an[d] / L[d] in ainv;
    // lawd: kLawD doubles per law cell (the truncated-normal laws of ALIGN_LAW 1)
    const float* law;
    const double* lawd;
    int32_t an[3];
    float ainv[3];
};

// One orientation law: rotation m[9] (row-major, applied to the drawn
// direction; column 2 is the law's axis), kappa, exp(-2 kappa), sampling
// flags (bit 0: von Mises-Fisher with that kappa, else isotropic; bit 1:
// rotate the draw by m; bit 2: theta / phi drawn by the cell's own
// truncated-normal laws where the realisation's law draws them so), the
// cell's median theta and phi. kappa > 0 with bit 0 clear: a fitted law that
// only the thin-out uses. The doubles of a cell: theta median and scale, phi
// median and scale, then (c1, c2, zmax) of tn_angle for theta and for phi.
constexpr int kLawF = 14;
constexpr int kLawD = 10;

// Law cell of a point: floor(x an / L) per axis, clamped to the grid.
NF_HD uint32_t law_cell(const Real& R, float x, float y, float z) {
    int c[3];
    const float v[3] = {x, y, z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int i = (int)fmul(v[d], R.ainv[d]);
        c[d] = i < 0 ? 0 : (i >= R.an[d] ? R.an[d] - 1 : i);
    }
    return (uint32_t)(c[0] + R.an[0] * (c[1] + R.an[1] * c[2]));
}

NF_HD float lerp_nf(float a, float b, float f) { return fadd(a, fmul(fsub(b, a), f)); }

// Trilinear density with wrap addressing, texel centres at (i+0.5)/n
// (the texture set-up of inc/den2tex.h:36-40, evaluated in full FP32).
NF_HD float density(const Real& R, float x, float y, float z) {
    if (!R.mesh) return R.dflt;
    float pos[3] = {x, y, z};
    int i0[3], i1[3];
    float f[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float g = fsub(fmul(fdiv(pos[d], R.L[d]), (float)R.mn[d]), 0.5f);
        float fl = floorf(g);
        f[d] = fsub(g, fl);
        int i = (int)fl;
        i %= R.mn[d];
        if (i < 0) i += R.mn[d];
        i0[d] = i;
        i1[d] = (i + 1 == R.mn[d]) ? 0 : i + 1;
    }
    const int ny = R.mn[1], nz = R.mn[2];
#define NF_V(i, j, k) R.mesh[((size_t)(i) * ny + (j)) * nz + (k)]
    float c00 = lerp_nf(NF_V(i0[0], i0[1], i0[2]), NF_V(i1[0], i0[1], i0[2]), f[0]);
    float c10 = lerp_nf(NF_V(i0[0], i1[1], i0[2]), NF_V(i1[0], i1[1], i0[2]), f[0]);
    float c01 = lerp_nf(NF_V(i0[0], i0[1], i1[2]), NF_V(i1[0], i0[1], i1[2]), f[0]);
    float c11 = lerp_nf(NF_V(i0[0], i1[1], i1[2]), NF_V(i1[0], i1[1], i1[2]), f[0]);
#undef NF_V
    float c0 = lerp_nf(c00, c10, f[1]);
    float c1 = lerp_nf(c01, c11, f[1]);
    return lerp_nf(c0, c1, f[2]);
}

// Candidate k of the stream: pos = (x,y,z,l), dir = (cx,cy,cz,a), u, rho.
NF_HD void candidate(const Real& R, uint64_t k, float4* pos, float4* dir, float* u, float* rho) {
    const uint32_t klo = (uint32_t)k, khi = (uint32_t)(k >> 32);
    U4 A = philox(klo, khi, 0u, 0u, R.key[0], R.key[1]);
    U4 B = philox(klo, khi, 1u, 0u, R.key[0], R.key[1]);
    float x = fmul(uni(A.x), R.L[0]);
    float y = fmul(uni(A.y), R.L[1]);
    float z = fmul(uni(A.z), R.L[2]);
    float uu = uni(A.w);
    // the law of the realisation, or of the candidate's law cell
    const float* m = R.m;
    float kappa = R.kappa, E2 = R.E2;
    bool vmf = R.orient == 1, rot = R.rot != 0;
    float tmed = R.tmed, pmed = R.pmed;
    double tc1 = R.tc1, tc2 = R.tc2, tz = R.tz, pc1 = R.pc1, pc2 = R.pc2, pz = R.pz;
    if (R.law) {
        const uint32_t lc = law_cell(R, x, y, z);
        const float* Lw = R.law + (size_t)kLawF * lc;
        m = Lw;
        kappa = Lw[9];
        E2 = Lw[10];
        const int fl = (int)Lw[11];
        vmf = (fl & 1) != 0;
        rot = (fl & 2) != 0;
        if (fl & 4) {  // the cell's truncated-normal laws
            const double* Ld = R.lawd + (size_t)kLawD * lc;
            tmed = Lw[12];
            pmed = Lw[13];
            tc1 = Ld[4]; tc2 = Ld[5]; tz = Ld[6];
            pc1 = Ld[7]; pc2 = Ld[8]; pz = Ld[9];
        }
    }
    float cz;
    if (vmf) {
        float w = fsub(1.0f, uni(B.x));
        float v = fadd(w, fmul(fsub(1.0f, w), E2));
        cz = fadd(1.0f, fdiv(log_nf(v), kappa));
        cz = cz < -1.0f ? -1.0f : (cz > 1.0f ? 1.0f : cz);
    } else if (R.tn & 1) {  // genCosine: cos of a truncated-normal theta
        const double th = tn_angle(uni(B.x), tmed, tc1, tc2, tz);
        float st;
        sincos_turns((float)dmul(th, kInv2PiD), &cz, &st);
    } else {
        cz = fsub(fmul(uni(B.x), 2.0f), 1.0f);
    }
    float cp, sp;
    if (R.tn & 2) {  // truncated-normal phi
        const double ph = tn_angle(uni(B.y), pmed, pc1, pc2, pz);
        sincos_turns((float)dmul(ph, kInv2PiD), &cp, &sp);
    } else {
        sincos_turns(uni(B.y), &cp, &sp);
    }
    float sr = fsub(1.0f, fmul(cz, cz));
    float s = fsqrt(sr > 0.0f ? sr : 0.0f);
    float cx = fmul(s, cp), cy = fmul(s, sp);
    if (rot) {
        float rx = fadd(fadd(fmul(m[0], cx), fmul(m[1], cy)), fmul(m[2], cz));
        float ry = fadd(fadd(fmul(m[3], cx), fmul(m[4], cy)), fmul(m[5], cz));
        float rz = fadd(fadd(fmul(m[6], cx), fmul(m[7], cy)), fmul(m[8], cz));
        cx = rx; cy = ry; cz = rz;
    }
    float len = R.l;
    if (R.len_mode == 1) {
        float cb, sb;
        sincos_turns(uni(B.w), &cb, &sb);
        float g = fmul(fsqrt(fmul(-2.0f, log_nf(fsub(1.0f, uni(B.z))))), cb);
        len = fmul(R.l, exp_nf(fmul(R.sigma, g)));
        len = len < R.lmin ? R.lmin : (len > R.lmax ? R.lmax : len);
    }
    float rad = R.a;
    if (R.rad_mode == 2) {
        U4 Cc = philox(klo, khi, 2u, 0u, R.key[0], R.key[1]);
        rad = fadd(R.rmin, fmul(fsub(R.rmax, R.rmin), uni(Cc.x)));
    }
    *pos = make_float4(x, y, z, len);
    *dir = make_float4(cx, cy, cz, rad);
    *u = uu;
    *rho = density(R, x, y, z);
}

// ---------------------------------------------------------------------------
// Cells.
// ---------------------------------------------------------------------------
NF_HD int cell_coord(const Real& R, int d, float x) {
    int c = (int)(x * R.invE[d]);
    if (x < 0.0f) c = -1;
    c = c < 0 ? 0 : (c >= R.n[d] ? R.n[d] - 1 : c);
    return c;
}

NF_HD uint32_t cell_of(const Real& R, float x, float y, float z) {
    int cx = cell_coord(R, 0, x), cy = cell_coord(R, 1, y), cz = cell_coord(R, 2, z);
    return R.cell_off + (uint32_t)(cx + R.n[0] * (cy + R.n[1] * cz));
}

// Row r of the (2S+1)^2 rows of the stencil of cell c: the cells at
// (c.x - S .. c.x + S, c.y + dy, c.z + dz). Along x the row is split where it
// wraps, into at most 3 runs of consecutive cells, each with one periodic image.
// Returns the number of runs (0 when the row leaves an open axis).
struct Run {
    uint32_t lo, hi;  // global ids of the first and last cell of the run
    int img[3];
};

NF_HD int stencil_row(const Real& R, const int c[3], int r, int per, Run run[3]) {
    const int w = 2 * R.S + 1;
    if (r >= w * w) return 0;
    int q[3], im[3] = {0, 0, 0};
    const int off[3] = {0, r % w - R.S, r / w - R.S};
#pragma unroll
    for (int d = 1; d < 3; ++d) {
        int v = c[d] + off[d];
        if (v < 0) {
            if (!(per & (1 << d))) return 0;
            v += R.n[d]; im[d] = -1;
        } else if (v >= R.n[d]) {
            if (!(per & (1 << d))) return 0;
            v -= R.n[d]; im[d] = 1;
        }
        q[d] = v;
    }
    const uint32_t base = R.cell_off + (uint32_t)(R.n[0] * (q[1] + R.n[1] * q[2]));
    const int nx = R.n[0], x0 = c[0] - R.S, x1 = c[0] + R.S;
    const bool px = (per & 1) != 0;
    int k = 0;
    auto put = [&](int lo, int hi, int ix) {
        run[k].lo = base + (uint32_t)lo;
        run[k].hi = base + (uint32_t)hi;
        run[k].img[0] = ix; run[k].img[1] = im[1]; run[k].img[2] = im[2];
        ++k;
    };
    if (px && x0 < 0) put(x0 + nx, nx - 1, -1);
    put(x0 < 0 ? 0 : x0, x1 >= nx ? nx - 1 : x1, 0);
    if (px && x1 >= nx) put(0, x1 - nx, 1);
    return k;
}

// ---------------------------------------------------------------------------
// FP32 conservative filter. The reference's points lie on the two axis lines,
// within (l/2 + a + eps)|c| of each centre, so d is bounded below by
//   (1) the centre distance minus both half-reaches (bounding spheres),
//   (2) the distance of the two lines, |(cA x cB) . b| / |cA x cB|,
//   (3) the gap of the projections of the two segments onto cA, and onto cB
//       (projection is 1-Lipschitz: a separating-axis bound).
// A pair is "far" when one bound, evaluated in FP32 with error margins
// (relative 2e-6 .. 2e-4, absolute `slack` for coordinate rounding), clears the
// threshold; far pairs cannot satisfy d < thr in any precision. The rest go to
// the FP64 routine.
// ---------------------------------------------------------------------------
NF_HD bool maybe_near(const float4& pA, const float4& cA, const float4& pB, const float4& cB, float sx, float sy,
                      float sz, float thr, float eps, float slack) {
    float bx = (pB.x + sx) - pA.x, by = (pB.y + sy) - pA.y, bz = (pB.z + sz) - pA.z;
    float hA = pA.w * 0.5f + cA.w + eps, hB = pB.w * 0.5f + cB.w + eps;
    float Rr = (hA + hB + thr) * 1.000002f + slack;
    float bb = bx * bx + by * by + bz * bz;
    if (bb > Rr * Rr) return false;
    float err = 4e-6f * (1.0f + sqrtf(bb)) + slack;
    float thr_s = thr * 1.0002f;
    float dcc = fabsf(cA.x * cB.x + cA.y * cB.y + cA.z * cB.z);
    float pa = fabsf(bx * cA.x + by * cA.y + bz * cA.z);
    if (pa - (hA + hB * dcc) * 1.00001f - err > thr_s) return false;
    float pb = fabsf(bx * cB.x + by * cB.y + bz * cB.z);
    if (pb - (hB + hA * dcc) * 1.00001f - err > thr_s) return false;
    float nx = cA.y * cB.z - cA.z * cB.y;
    float ny = cA.z * cB.x - cA.x * cB.z;
    float nz = cA.x * cB.y - cA.y * cB.x;
    float nn = nx * nx + ny * ny + nz * nz;
    if (nn > 1e-4f) {
        float nb = fabsf(nx * bx + ny * by + nz * bz);
        float s = sqrtf(nn);
        if (nb - err > thr_s * s) return false;
    }
    // (4) separating axis through approximate closest points of the two
    // extended segments: for any direction u, min over B of u.x - max over A
    // of u.x bounds d from below (the reference's points lie on these
    // segments); u from the clamped closest points (Ericson, Real-Time
    // Collision Detection, 5.1.9) makes the bound nearly tight, and how
    // accurate those points are does not matter for its validity. Catches
    // segments whose lines pass close but whose ends stay apart.
    {
        const float ha = hA * 1.00001f, hb = hB * 1.00001f;
        const float d1x = 2.0f * ha * cA.x, d1y = 2.0f * ha * cA.y, d1z = 2.0f * ha * cA.z;
        const float d2x = 2.0f * hb * cB.x, d2y = 2.0f * hb * cB.y, d2z = 2.0f * hb * cB.z;
        const float a0x = -ha * cA.x, a0y = -ha * cA.y, a0z = -ha * cA.z;  // A from a0 to a0 + d1
        const float b0x = bx - hb * cB.x, b0y = by - hb * cB.y, b0z = bz - hb * cB.z;  // B from b0 to b0 + d2
        const float rx = a0x - b0x, ry = a0y - b0y, rz = a0z - b0z;
        const float a = d1x * d1x + d1y * d1y + d1z * d1z, e = d2x * d2x + d2y * d2y + d2z * d2z;
        const float f = d2x * rx + d2y * ry + d2z * rz, c = d1x * rx + d1y * ry + d1z * rz;
        const float bq = d1x * d2x + d1y * d2y + d1z * d2z;
        const float den = a * e - bq * bq;
        float sA = den > 1e-12f * a * e ? fminf(fmaxf((bq * f - c * e) / den, 0.0f), 1.0f) : 0.0f;
        float tB = e > 0.0f ? (bq * sA + f) / e : 0.0f;
        if (tB < 0.0f) { tB = 0.0f; sA = a > 0.0f ? fminf(fmaxf(-c / a, 0.0f), 1.0f) : 0.0f; }
        else if (tB > 1.0f) { tB = 1.0f; sA = a > 0.0f ? fminf(fmaxf((bq - c) / a, 0.0f), 1.0f) : 0.0f; }
        const float ux = (b0x + d2x * tB) - (a0x + d1x * sA);
        const float uy = (b0y + d2y * tB) - (a0y + d1y * sA);
        const float uz = (b0z + d2z * tB) - (a0z + d1z * sA);
        const float nu = sqrtf(ux * ux + uy * uy + uz * uz);
        if (nu > 1e-12f) {
            const float pa0 = ux * a0x + uy * a0y + uz * a0z;
            const float pa1 = pa0 + (ux * d1x + uy * d1y + uz * d1z);
            const float pb0 = ux * b0x + uy * b0y + uz * b0z;
            const float pb1 = pb0 + (ux * d2x + uy * d2y + uz * d2z);
            const float sep = (fminf(pb0, pb1) - fmaxf(pa0, pa1)) / nu;
            if (sep * 0.99999f - err - 4e-6f * (ha + hb) > thr_s) return false;
        }
    }
    return true;
}

// The line-distance test of maybe_near on its own (same expressions, so
// line_far() true implies maybe_near() false): the two infinite axis lines are
// certainly farther apart than thr. Near-parallel pairs are never far here.
NF_HD bool line_far(const float4& pA, const float4& cA, const float4& pB, const float4& cB, float sx, float sy,
                    float sz, float thr, float slack) {
    float bx = (pB.x + sx) - pA.x, by = (pB.y + sy) - pA.y, bz = (pB.z + sz) - pA.z;
    float bb = bx * bx + by * by + bz * bz;
    float nx = cA.y * cB.z - cA.z * cB.y;
    float ny = cA.z * cB.x - cA.x * cB.z;
    float nz = cA.x * cB.y - cA.y * cB.x;
    float nn = nx * nx + ny * ny + nz * nz;
    if (!(nn > 1e-4f)) return false;
    float err = 4e-6f * (1.0f + sqrtf(bb)) + slack;
    float nb = fabsf(nx * bx + ny * by + nz * bz);
    return nb - err > thr * 1.0002f * sqrtf(nn);
}

// The sphere bound of maybe_near with the probe's terms hoisted: hAs = hA +
// thr-part of A, evaluated once per probe; hB and aB staged with the target.
// Same inequality as the first test of maybe_near (conservative).
NF_HD bool sphere_far(float bx, float by, float bz, float hA_plus, float hB, float aB, float scf, float slack) {
    float Rr = (hA_plus + hB + aB * scf) * 1.000002f + slack;
    return bx * bx + by * by + bz * bz > Rr * Rr;
}

// FP32 certificate of a hit. When the reference routine takes its
// non-parallel branch and leaves both parameters unclamped (|t| <= l/2 + a + eps
// for both rods), its points are the feet of the common perpendicular and d is
// exactly the distance of the two lines. The certificate demands margins that
// exceed the FP32 error of every quantity involved: |c1.c2| <= 0.995 (so
// |d^2 - 1| >= 0.0099 and the branch is far from the 1e-6 parallel test), both
// |t| at least dt inside their limits, and the line distance at least err
// below the threshold. Certified pairs are hits in FP64 as well.
NF_HD bool certain_hit(const float4& pA, const float4& cA, const float4& pB, const float4& cB, float sx, float sy,
                       float sz, float thr, float eps, float slack, float* t0o = nullptr, float* t1o = nullptr) {
    float bx = (pB.x + sx) - pA.x, by = (pB.y + sy) - pA.y, bz = (pB.z + sz) - pA.z;
    float d = cA.x * cB.x + cA.y * cB.y + cA.z * cB.z;
    if (fabsf(d) > 0.995f) return false;
    float den = d * d - 1.0f;
    float nb = sqrtf(bx * bx + by * by + bz * bz);
    float t0 = ((d * cB.x - cA.x) * bx + (d * cB.y - cA.y) * by + (d * cB.z - cA.z) * bz) / den;
    float t1 = ((cB.x - d * cA.x) * bx + (cB.y - d * cA.y) * by + (cB.z - d * cA.z) * bz) / den;
    float dt = (2e-5f * (1.0f + nb) + 2.0f * slack) / fabsf(den);
    if (fabsf(t0) + dt >= (pA.w * 0.5f + cA.w + eps) * 0.99999f) return false;
    if (fabsf(t1) + dt >= (pB.w * 0.5f + cB.w + eps) * 0.99999f) return false;
    if (t0o) { *t0o = t0; *t1o = t1; }
    float nx = cA.y * cB.z - cA.z * cB.y;
    float ny = cA.z * cB.x - cA.x * cB.z;
    float nz = cA.x * cB.y - cA.y * cB.x;
    float s = sqrtf(nx * nx + ny * ny + nz * nz);
    float ld = fabsf(nx * bx + ny * by + nz * bz) / s;
    float err = (4e-6f * (1.0f + nb) + slack) / s + 1e-6f * ld;
    return ld + err < thr * 0.9998f;
}

// ---------------------------------------------------------------------------
// The reference routine in FP64, without contraction (matches the oracle).
// A in "registers", B shifted by (sx,sy,sz). Returns d; t0,t1 clamped;
// u0,u1 unclamped; Dx the perpendicular distance at (u0,u1).
// ---------------------------------------------------------------------------
struct RodD { double x, y, z, cx, cy, cz, l, a; };

NF_HD RodD rodd(const float4& p, const float4& c) {
    return RodD{(double)p.x, (double)p.y, (double)p.z, (double)c.x, (double)c.y, (double)c.z,
                (double)p.w, (double)c.w};
}

NF_HD double ref_distance_d(const RodD& A, const RodD& B, double sx, double sy, double sz,
                            double eps, bool typo, double* t0o, double* t1o, double* u0o,
                            double* u1o, double* Dxo) {
    const double Bx = dadd(B.x, sx), By = dadd(B.y, sy), Bz = dadd(B.z, sz);
    const double bx = dsub(Bx, A.x), by = dsub(By, A.y), bz = dsub(Bz, A.z);
    double d = dadd(dadd(dmul(A.cx, B.cx), dmul(A.cy, B.cy)), dmul(A.cz, B.cz));
    double t0, t1;
    if (dsub(1.0, dabs(d)) > eps) {
        double ax = dsub(dmul(d, B.cx), A.cx), ay = dsub(dmul(d, B.cy), A.cy), az = dsub(dmul(d, B.cz), A.cz);
        t0 = dadd(dadd(dmul(ax, bx), dmul(ay, by)), dmul(az, bz));
        ax = dsub(B.cx, dmul(d, A.cx)); ay = dsub(B.cy, dmul(d, A.cy)); az = dsub(B.cz, dmul(d, A.cz));
        t1 = dadd(dadd(dmul(ax, bx), dmul(ay, by)), dmul(az, bz));
        double den = dsub(dmul(d, d), 1.0);
        t0 = ddiv(t0, den);
        t1 = ddiv(t1, den);
    } else {
        t0 = copysign(ddiv(A.l, 2.0), dadd(dadd(dmul(bx, A.cx), dmul(by, A.cy)), dmul(bz, A.cz)));
        double dot = typo ? dadd(dadd(dmul(bx, B.cx), dmul(bx, B.cy)), dmul(bx, B.cz))
                          : dadd(dadd(dmul(bx, B.cx), dmul(by, B.cy)), dmul(bz, B.cz));
        t1 = dadd(dmul(-1.0, dot), dmul(d, t0));
    }
    const double u0 = t0, u1 = t1;
    const double hA = ddiv(A.l, 2.0), hB = ddiv(B.l, 2.0);
    bool f1 = dabs(t0) <= dadd(dadd(hA, A.a), eps);
    bool f2 = dabs(t1) <= dadd(dadd(hB, B.a), eps);
    if (!(f1 && f2)) {
        bool f3 = dsub(dabs(t0), hA) < dsub(dabs(t1), hB);
        if (f3) {
            t1 = copysign(hB, t1);
            t0 = dadd(dmul(1.0, dadd(dadd(dmul(bx, A.cx), dmul(by, A.cy)), dmul(bz, A.cz))), dmul(d, t1));
            if (dabs(t0) > hA) t0 = copysign(hA, t0);
        } else {
            t0 = copysign(hA, t0);
            t1 = dadd(dmul(-1.0, dadd(dadd(dmul(bx, B.cx), dmul(by, B.cy)), dmul(bz, B.cz))), dmul(d, t0));
            if (dabs(t1) > hB) t1 = copysign(hB, t1);
        }
    }
    double px = dsub(dsub(dadd(A.x, dmul(t0, A.cx)), Bx), dmul(t1, B.cx));
    double py = dsub(dsub(dadd(A.y, dmul(t0, A.cy)), By), dmul(t1, B.cy));
    double pz = dsub(dsub(dadd(A.z, dmul(t0, A.cz)), Bz), dmul(t1, B.cz));
    double dist = dsqrt(dadd(dadd(dmul(px, px), dmul(py, py)), dmul(pz, pz)));
    if (Dxo) {
        double qx = dsub(dsub(dadd(A.x, dmul(u0, A.cx)), Bx), dmul(u1, B.cx));
        double qy = dsub(dsub(dadd(A.y, dmul(u0, A.cy)), By), dmul(u1, B.cy));
        double qz = dsub(dsub(dadd(A.z, dmul(u0, A.cz)), Bz), dmul(u1, B.cz));
        *Dxo = dsqrt(dadd(dadd(dmul(qx, qx), dmul(qy, qy)), dmul(qz, qz)));
    }
    if (t0o) *t0o = t0;
    if (t1o) *t1o = t1;
    if (u0o) *u0o = u0;
    if (u1o) *u1o = u1;
    return dist;
}

// (a_B + a_A) * scf + sep + eps, left to right (inc/intersection_dev.h:78).
NF_HD double thresh_d(double aA, double aB, double scf, double sep, double eps) {
    return dadd(dadd(dmul(dadd(aB, aA), scf), sep), eps);
}

// The same routine in plain FP32 (what an FP32-only build decides), for the
// would-flip diagnostic of the precision form.
__device__ __forceinline__ bool ref_hit_f32(const float4& pA, const float4& cA, const float4& pB,
                                            const float4& cB, float sx, float sy, float sz,
                                            float eps, float thr, bool typo) {
    float Bx = pB.x + sx, By = pB.y + sy, Bz = pB.z + sz;
    float bx = Bx - pA.x, by = By - pA.y, bz = Bz - pA.z;
    float d = cA.x * cB.x + cA.y * cB.y + cA.z * cB.z;
    float t0, t1;
    if (1.0f - fabsf(d) > eps) {
        float ax = d * cB.x - cA.x, ay = d * cB.y - cA.y, az = d * cB.z - cA.z;
        t0 = ax * bx + ay * by + az * bz;
        ax = cB.x - d * cA.x; ay = cB.y - d * cA.y; az = cB.z - d * cA.z;
        t1 = ax * bx + ay * by + az * bz;
        t0 /= d * d - 1.0f;
        t1 /= d * d - 1.0f;
    } else {
        t0 = copysignf(pA.w * 0.5f, bx * cA.x + by * cA.y + bz * cA.z);
        t1 = typo ? -(bx * cB.x + bx * cB.y + bx * cB.z) + d * t0 : -(bx * cB.x + by * cB.y + bz * cB.z) + d * t0;
    }
    float hA = pA.w * 0.5f, hB = pB.w * 0.5f;
    bool f1 = fabsf(t0) <= hA + cA.w + eps, f2 = fabsf(t1) <= hB + cB.w + eps;
    if (!(f1 && f2)) {
        bool f3 = (fabsf(t0) - hA) < (fabsf(t1) - hB);
        if (f3) {
            t1 = copysignf(hB, t1);
            t0 = (bx * cA.x + by * cA.y + bz * cA.z) + d * t1;
            if (fabsf(t0) > hA) t0 = copysignf(hA, t0);
        } else {
            t0 = copysignf(hA, t0);
            t1 = -(bx * cB.x + by * cB.y + bz * cB.z) + d * t0;
            if (fabsf(t1) > hB) t1 = copysignf(hB, t1);
        }
    }
    float px = pA.x + t0 * cA.x - Bx - t1 * cB.x;
    float py = pA.y + t0 * cA.y - By - t1 * cB.y;
    float pz = pA.z + t0 * cA.z - Bz - t1 * cB.z;
    return sqrtf(px * px + py * py + pz * pz) < thr;
}

// Realisation owning slot s, given the prefix table off[0..R] (off[0] = 0).
__device__ __forceinline__ int find_real(const uint32_t* off, int R, uint32_t s) {
    int lo = 0, hi = R;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= s) lo = mid; else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Warp-aggregated counters.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void warp_add_u64(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

}  // namespace nf
