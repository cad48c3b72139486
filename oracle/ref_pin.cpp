// ref_pin.cpp -- host wrapper around the reference's own geometric routines
// (TEST INFRASTRUCTURE). oracle/ref_build.sh compiles it with -I pointing at
// the reference's inc/ directory; nothing here is a copy of reference code.
// The outputs become golden vectors (tests/golden/) that pin the oracle's
// FP32 restatement bit for bit.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdlib>
// Host stand-ins for the CUDA device overloads the headers rely on: mixed
// float/double max/min promote to double, and blockDim exists (unused here).
static inline float max(float a, float b) { return fmaxf(a, b); }
static inline double max(float a, double b) { return fmax((double)a, b); }
static inline double max(double a, float b) { return fmax(a, (double)b); }
static inline double max(double a, double b) { return fmax(a, b); }
static inline float min(float a, float b) { return fminf(a, b); }
static inline double min(float a, double b) { return fmin((double)a, b); }
static inline double min(double a, float b) { return fmin(a, (double)b); }
static const dim3 blockDim(1, 1, 1);
#include "definitions.h"
#include "vectorMath.h"
#include "CNT.h"
#include "intersection_dev.h"
#include "intersect/intersect_cylinder_capped.h"

extern "C" {

// cnt_intersec_shr (inc/intersection_dev.h:10-80); A = probe, B = partner.
int ref_hardcore(const float* A, const float* B, float eps, float sep, float scf) {
    CNT_t probe;
    float a[9];
    for (int i = 0; i < 9; ++i) a[i] = A[i];
    make_INC(&probe, a);
    float shr[9];
    for (int i = 0; i < 9; ++i) shr[i] = B[i];
    return cnt_intersec_shr(probe, shr, 1, 0, eps, sep, scf) ? 1 : 0;
}

// distance_cylinder_capped + if_intersects_cylinder_capped
// (inc/intersect/intersect_cylinder_capped.h:69-159).
int ref_contact(const float* A, const float* B, float separation, float soft_frac, float* out6) {
    float reg[9], shr[9];
    for (int i = 0; i < 9; ++i) { reg[i] = A[i]; shr[i] = B[i]; }
    float3 Dtt;
    float3 dtt = distance_cylinder_capped(reg, shr, 1, 0, &Dtt);
    out6[0] = dtt.x; out6[1] = dtt.y; out6[2] = dtt.z;
    out6[3] = Dtt.x; out6[4] = Dtt.y; out6[5] = Dtt.z;
    return if_intersects_cylinder_capped(dtt.x, reg, shr, 1, 0, separation, soft_frac) ? 1 : 0;
}

// body_intersect_cylinder_capped (:181-183) on partner B at parameter t.
int ref_body(const float* B, float t) {
    float shr[9];
    for (int i = 0; i < 9; ++i) shr[i] = B[i];
    return body_intersect_cylinder_capped(t, shr, 1, 0) ? 1 : 0;
}

// surf_to_cylinder_capped (:204-293): A = probe, B = partner already at its image.
float ref_surface(const float* A, const float* B, const float* Dtt3, float rlim) {
    float reg[9], shr[9];
    for (int i = 0; i < 9; ++i) { reg[i] = A[i]; shr[i] = B[i]; }
    return surf_to_cylinder_capped(reg, shr, 1, 0, make_float3(Dtt3[0], Dtt3[1], Dtt3[2]), rlim);
}

// get_relative_crd (inc/vectorMath.h:283-305).
void ref_relative(const float* A, const float* B, const float* L, float* out) {
    float3 r = get_relative_crd(make_float3(A[0], A[1], A[2]), make_float3(B[0], B[1], B[2]),
                                make_float3(L[0], L[1], L[2]));
    out[0] = r.x; out[1] = r.y; out[2] = r.z;
}
}
