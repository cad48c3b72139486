// nf_bcr.cuh -- direct network solve by block cyclic reduction, one CTA per
// realisation.
//
// Replaces, on the device, the sparse direct solve of the offline Kirchhoff
// tool (tools/kirchhoff/kirchhoff.py:246-269, MKL DSS through zsolve_dss_sy,
// tools/kirchhoff/lib/solver.cpp:185-269) for networks whose reverse
// Cuthill-McKee band is at most 32 wide.
//
// With the unknowns in band order and cut into blocks of 32, a band of width
// <= 32 makes the matrix block tridiagonal: block i couples only to blocks
// i - 1 and i + 1. Odd-even reduction eliminates, level after level, every
// second block still present (stride s = 1, 2, 4, ...: the blocks
// i = s mod 2s), which is block Gaussian elimination in a nested-dissection
// order of the block chain: the Schur complement of a symmetric positive
// definite matrix stays symmetric positive definite, so no pivoting is needed.
// Eliminating block i with neighbours p = i - s and q = i + s:
//     D_i = L_i Delta_i L_i^T         (LDL^T in one warp, L_i unit lower)
//     Vl_i = L_i^-1 A[i][p],  Vr_i = L_i^-1 A[i][q]
//     D_p -= Vl_i^T Delta_i^-1 Vl_i,  D_q -= Vr_i^T Delta_i^-1 Vr_i
//     A[q][p] = -Vr_i^T Delta_i^-1 Vl_i           (p and q become neighbours)
// Every block still present at a level is one warp's task: the updates its
// diagonal block receives from the eliminations of the level below, then its
// own elimination; one block barrier per level, log2(blocks) + 1 levels
// against one sequential pivot per unknown for a banded LDL^T. The solves go
// through the same levels: forward (w_i = Delta_i^-1 L_i^-1 r_i, neighbours
// lose Vl/Vr^T w_i), the last block, and back
// (x_i = L_i^-T (w_i - Delta_i^-1 (Vl_i x_p + Vr_i x_q))). L_i^-1 is formed
// explicitly, so every step of a solve is a 32 x 32 matrix-vector product.
//
// Blocks are row-major 32 x 32 arrays; a warp holds a block by columns (lane
// j: column j) or a block vector by elements (lane r: element r).
#pragma once

#include <cstdint>

namespace nf {

constexpr uint32_t kBcrW = 32;                    // block edge; the band must not be wider
constexpr uint32_t kBcrBlk = kBcrW * kBcrW;       // entries of one block
constexpr size_t kBcrPer = 8 * (size_t)kBcrBlk + kBcrW;  // D, K, Li, Lr, Vl, Vr, VlT, VrT, g per block

// Storage of block i: D (diagonal block, Schur-updated), K (A[i][left
// neighbour], updated as neighbours are eliminated), Li ((L_i^-1)^T) and Lr
// (L_i^-1), Vl, Vr and their transposes, g (inverse pivots 1 / Delta). Each
// product of a solve reads one of them by columns (coalesced).
template <typename T>
struct BcrBlock {
    T *D, *K, *Li, *Lr, *Vl, *Vr, *VlT, *VrT, *g;
};

template <typename T>
__device__ __forceinline__ BcrBlock<T> bcr_block(T* base, uint32_t i) {
    T* p = base + (size_t)i * kBcrPer;
    return {p,
            p + kBcrBlk,
            p + 2 * kBcrBlk,
            p + 3 * kBcrBlk,
            p + 4 * kBcrBlk,
            p + 5 * kBcrBlk,
            p + 6 * kBcrBlk,
            p + 7 * kBcrBlk,
            p + 8 * kBcrBlk};
}

// v[a] = M[a][lane] (column `lane`; one coalesced row per a)
template <typename T>
__device__ __forceinline__ void bcr_ld_col(const T* M, int lane, T (&v)[32]) {
#pragma unroll
    for (int a = 0; a < 32; ++a) v[a] = M[a * 32 + lane];
}

template <typename T>
__device__ __forceinline__ void bcr_st_col(T* M, int lane, const T (&v)[32]) {
#pragma unroll
    for (int a = 0; a < 32; ++a) M[a * 32 + lane] = v[a];
}

// v[a] = M[lane][a] (row `lane`, 16-byte loads; blocks are 16-byte aligned)
__device__ __forceinline__ void bcr_ld_row(const float* M, int lane, float (&v)[32]) {
    const float4* p = reinterpret_cast<const float4*>(M + lane * 32);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float4 x = p[q];
        v[4 * q] = x.x;
        v[4 * q + 1] = x.y;
        v[4 * q + 2] = x.z;
        v[4 * q + 3] = x.w;
    }
}

__device__ __forceinline__ void bcr_ld_row(const double* M, int lane, double (&v)[32]) {
    const double2* p = reinterpret_cast<const double2*>(M + lane * 32);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        const double2 x = p[q];
        v[2 * q] = x.x;
        v[2 * q + 1] = x.y;
    }
}

// M[lane][a] = v[a] (row `lane`, 16-byte stores)
__device__ __forceinline__ void bcr_st_row(float* M, int lane, const float (&v)[32]) {
    float4* p = reinterpret_cast<float4*>(M + lane * 32);
#pragma unroll
    for (int q = 0; q < 8; ++q) p[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

__device__ __forceinline__ void bcr_st_row(double* M, int lane, const double (&v)[32]) {
    double2* p = reinterpret_cast<double2*>(M + lane * 32);
#pragma unroll
    for (int q = 0; q < 16; ++q) p[q] = make_double2(v[2 * q], v[2 * q + 1]);
}

// In-register LDL^T of the symmetric block held by columns in c. On return
// c[t] (t > lane) holds the unscaled column A^(lane)[t][lane], c[lane] the
// pivot, *inv its inverse; false when a pivot is not a positive finite number.
template <typename T>
__device__ __forceinline__ bool bcr_ldl(T (&c)[32], int lane, T* inv) {
    bool ok = true;
    T my = 0;
#pragma unroll
    for (int k = 0; k < 32; ++k) {
        const T dk = __shfl_sync(0xffffffffu, c[k], k);
        ok = ok && dk > T(0) && dk < T(INFINITY);
        const T ik = T(1) / dk;
        if (lane == k) my = ik;
        const T f = c[k] * ik;  // A[k][lane] / pivot (the column's own copy of the symmetric entry)
#pragma unroll
        for (int t = 0; t < 32; ++t) {  // a constant trip count keeps both loops unrolled
            if (t > k) {
                const T a = __shfl_sync(0xffffffffu, c[t], k);
                if (lane > k) c[t] -= a * f;
            }
        }
    }
    *inv = my;
    return ok;
}

// Each warp's shared scratch: S (32 x 32), S2 (32 x 33, padded so that a
// lane can read a row while the warp writes columns) and Sg (32).
constexpr uint32_t kBcrScratch = kBcrBlk + 32 * 33 + 32;

// 32 consecutive shared values from p (16-byte aligned) into v
__device__ __forceinline__ void bcr_ld_sh(const float* p, float (&v)[32]) { bcr_ld_row(p, 0, v); }
__device__ __forceinline__ void bcr_ld_sh(const double* p, double (&v)[32]) { bcr_ld_row(p, 0, v); }

// S <- (L^-1)^T (row-major), for the factor in c (see bcr_ldl); x = row
// `lane` of L^-1, so S[t][lane] = x[t]. S is first used for L itself.
template <typename T>
__device__ __forceinline__ void bcr_linv(const T (&c)[32], T inv, int lane, T* S, T (&x)[32]) {
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 32; ++t) S[t * 32 + lane] = t > lane ? c[t] * inv : T(t == lane ? 1 : 0);
    __syncwarp();
    // x^T L = e_lane^T: x[t] = [t == lane] - sum_{a > t} L[a][t] x[a] (x[a] = 0 for a > lane)
#pragma unroll
    for (int t = 31; t >= 0; --t) {
        T acc = t == lane ? T(1) : T(0);
#pragma unroll
        for (int a = t + 1; a < 32; ++a) acc -= S[a * 32 + t] * x[a];
        x[t] = acc;
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < 32; ++t) S[t * 32 + lane] = x[t];
    __syncwarp();
}

// v = L^-1 m for the column m of a block, (L^-1)^T in S
template <typename T>
__device__ __forceinline__ void bcr_lmul(const T* S, const T (&m)[32], T (&v)[32]) {
#pragma unroll
    for (int a = 0; a < 32; ++a) v[a] = 0;
#pragma unroll
    for (int r = 0; r < 32; ++r) {
        T row[32];
        bcr_ld_sh(S + r * 32, row);  // L^-1[a][r] over a (zero above the diagonal)
#pragma unroll
        for (int a = r; a < 32; ++a) v[a] += row[a] * m[r];
    }
}

// d[a] -= sum_k S[k][a] Sg[k] S[k][lane]: column `lane` of S^T G S with
// G = diag(Sg) (S and Sg hold V and g)
template <typename T>
__device__ __forceinline__ void bcr_sub_vgv(const T* S, const T* Sg, int lane, T (&d)[32]) {
#pragma unroll 4
    for (int k = 0; k < 32; ++k) {
        const T vk = S[k * 32 + lane] * Sg[k];
        T row[32];
        bcr_ld_sh(S + k * 32, row);
#pragma unroll
        for (int a = 0; a < 32; ++a) d[a] -= row[a] * vk;
    }
}

// d -= V^T diag(g) V for the column `lane` d of a diagonal block; V, g in
// global memory
template <typename T>
__device__ __forceinline__ void bcr_schur(const T* V, const T* g, int lane, T* S, T* Sg, T (&d)[32]) {
    T v[32];
    bcr_ld_col(V, lane, v);  // every load in flight at once
    const T gl = g[lane];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 32; ++k) S[k * 32 + lane] = v[k];
    Sg[lane] = gl;
    __syncwarp();
    bcr_sub_vgv(S, Sg, lane, d);
}

// y_lane = sum_k M[k][lane] x_k
template <typename T>
__device__ __forceinline__ T bcr_mtv(const T* M, T x, int lane) {
    T acc = 0;
#pragma unroll
    for (int k = 0; k < 32; ++k) acc += M[k * 32 + lane] * __shfl_sync(0xffffffffu, x, k);
    return acc;
}

// Factorisation of the m blocks at base (D and K assembled); sc is the
// warp's scratch (kBcrScratch entries). Returns false (in every thread) when
// a pivot is not positive: the system is not positive definite at this
// precision.
template <int NT, typename T>
__device__ bool bcr_factor(T* base, uint32_t m, T* sc, int* bad) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T* S = sc;
    T* S2 = sc + kBcrBlk;
    T* Sg = S2 + 32 * 33;
    for (uint32_t s = 1;; s <<= 1) {
        const uint32_t h = s >> 1, ntask = (m - 1) / s + 1;
        for (uint32_t task = warp; task < ntask; task += NT / 32) {
            const uint32_t i = task * s;
            const bool elim = (task & 1u) && s < m;
            if (h == 0 && !elim && s < m) continue;  // level 0: only the eliminated blocks have work
            BcrBlock<T> B = bcr_block(base, i);
            T d[32];
            bcr_ld_col(B.D, lane, d);
            if (h) {  // the eliminations of the level below: blocks i - h and i + h
                if (i >= h) {
                    BcrBlock<T> P = bcr_block(base, i - h);
                    bcr_schur(P.Vr, P.g, lane, S, Sg, d);
                }
                if (i + h < m) {
                    BcrBlock<T> Q = bcr_block(base, i + h);
                    bcr_schur(Q.Vl, Q.g, lane, S, Sg, d);
                }
            }
            if (!elim && s < m) {  // present at the next level
                bcr_st_col(B.D, lane, d);
                continue;
            }
            T inv;
            if (!bcr_ldl(d, lane, &inv)) *bad = 1;
            {
                T x[32];
                bcr_linv(d, inv, lane, S, x);
                bcr_st_col(B.Li, lane, x);  // (L^-1)^T
                bcr_st_row(B.Lr, lane, x);  // L^-1
            }
            B.g[lane] = inv;
            if (!elim) continue;  // the last block
            T mm[32], v[32];
            bcr_ld_col(B.K, lane, mm);  // A[i][i - s], column `lane`
            bcr_lmul(S, mm, v);
            bcr_st_col(B.Vl, lane, v);
            bcr_st_row(B.VlT, lane, v);
            const uint32_t q = i + s;
            if (q < m) {
                BcrBlock<T> Q = bcr_block(base, q);
                __syncwarp();
#pragma unroll
                for (int k = 0; k < 32; ++k) S2[k * 33 + lane] = v[k];  // Vl, for the new coupling
                bcr_ld_row(Q.K, lane, mm);  // A[i][q] = A[q][i]^T: column `lane` is row `lane` of Q.K
                bcr_lmul(S, mm, v);
                bcr_st_col(B.Vr, lane, v);
                bcr_st_row(B.VrT, lane, v);
                __syncwarp();
#pragma unroll
                for (int k = 0; k < 32; ++k) S[k * 32 + lane] = v[k];  // Vr
                Sg[lane] = inv;
                __syncwarp();
                // A[q][p] = -Vr^T G Vl, column `lane`
#pragma unroll
                for (int a = 0; a < 32; ++a) v[a] = 0;
#pragma unroll 4
                for (int k = 0; k < 32; ++k) {
                    const T vk = S2[k * 33 + lane] * Sg[k];
                    T row[32];
                    bcr_ld_sh(S + k * 32, row);
#pragma unroll
                    for (int a = 0; a < 32; ++a) v[a] -= row[a] * vk;
                }
                bcr_st_col(Q.K, lane, v);
            }
        }
        __syncthreads();
        if (s >= m) break;
    }
    return *bad == 0;
}

// Solves in place for the right-hand side t (m blocks of 32, band order).
template <int NT, typename T>
__device__ void bcr_solve(T* base, uint32_t m, T* t) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t top = 1;  // smallest power of two >= m
    while (top < m) top <<= 1;
    for (uint32_t s = 1;; s <<= 1) {  // forward
        const uint32_t h = s >> 1, ntask = (m - 1) / s + 1;
        for (uint32_t task = warp; task < ntask; task += NT / 32) {
            const uint32_t i = task * s;
            const bool elim = (task & 1u) && s < m;
            if (h == 0 && !elim && s < m) continue;
            T tv = t[i * 32 + lane];
            if (h) {
                if (i >= h) tv -= bcr_mtv(bcr_block(base, i - h).Vr, t[(i - h) * 32 + lane], lane);
                if (i + h < m) tv -= bcr_mtv(bcr_block(base, i + h).Vl, t[(i + h) * 32 + lane], lane);
            }
            if (elim || s >= m) {  // Li holds (L^-1)^T, Lr L^-1
                BcrBlock<T> B = bcr_block(base, i);
                tv = bcr_mtv(B.Li, tv, lane) * B.g[lane];
                if (!elim) tv = bcr_mtv(B.Lr, tv, lane);  // the last block: x_0
            }
            t[i * 32 + lane] = tv;
        }
        __syncthreads();
        if (s >= m) break;
    }
    for (uint32_t s = top >> 1; s >= 1; s >>= 1) {  // back
        const uint32_t ntask = (m - 1) / s + 1;
        for (uint32_t task = 1 + 2 * (uint32_t)warp; task < ntask; task += 2 * (NT / 32)) {
            const uint32_t i = task * s;
            BcrBlock<T> B = bcr_block(base, i);
            T u = bcr_mtv(B.VlT, t[(i - s) * 32 + lane], lane);
            if (i + s < m) u += bcr_mtv(B.VrT, t[(i + s) * 32 + lane], lane);
            const T v = t[i * 32 + lane] - B.g[lane] * u;
            t[i * 32 + lane] = bcr_mtv(B.Lr, v, lane);
        }
        __syncthreads();
    }
}

}  // namespace nf
