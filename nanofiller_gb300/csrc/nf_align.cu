// nf_align.cu -- adaptive generation: per-cell orientation laws refit from the
// accepted rods (self-alignment), thin-out of the rods the new laws make
// unlikely, and clusterisation of new candidates onto older rods.
//
// The reference (src/cudaMain.cu:112-132, 254-273, 354-396):
//   - every SELF_ALLIGN_STEP rounds, or after a round that gained fewer than
//     1 % of the rods still missing, it builds per cell the orientation
//     tensor <c c^T> of the rods (crossMtxBuild, inc/allignment_fit.h:154-210),
//     takes an eigenvector of it as the cell's preferred axis (resetOrt,
//     :214-274) and the spread of the rods about it as the cell's law
//     (resetAvgVec, :353-458); later candidates of the cell draw their
//     direction from that law (cuda_CNTgenerate_orient,
//     inc/cuda_CNTgenerate.h:136-260);
//   - with REDUCE_FLAG it then deletes each rod with probability
//     1 - min(1, 2 F), F the rod's likelihood under its cell's law relative to
//     the law's mode (randomThinOut / check_probability, :463-578);
//   - with CLUST_FLAG each new candidate is compared, before any hard-core
//     test, with the older rods of the neighbour cells: when their centres are
//     closer than half the longer length, their axes within CLUST_ANGL_LIM and
//     their closest points within CLUST_DIST_LIM (cnt_minDist,
//     inc/intersection_dev.h:85-160), the candidate is moved parallel to the
//     older rod at distance a + a' + INC_SEPARATION from its axis
//     (cuda_Clusterize2Old, inc/cuda_Clusterize.h:14-100).
//
// GB300 form, deterministic and independent of the round sizes:
//   - the candidate stream is cut into epochs of EPOCH_CANDIDATES; a round
//     never crosses an epoch boundary; refits and thin-out happen at
//     boundaries, and clusterisation uses the rods present when the epoch
//     began;
//   - a cell's law is a von Mises-Fisher law (the sampler that replaces the
//     reference's truncated normal) about the principal axis of the cell's
//     orientation tensor, with the concentration whose second moment
//     E[(c.mu)^2] = 1 - 2 coth(k)/k + 2/k^2 equals the tensor's largest
//     eigenvalue; the tensor sums are exact integers (products of FP32
//     components are exact in FP64 and are rounded to 2^-40), so they do not
//     depend on the order of the atomics; the 3x3 eigenproblems and the
//     concentrations are solved on the host in FP64 (cyclic Jacobi; bisection);
//   - thin-out: keep a rod when 2 exp(kappa (|c.mu| - 1)) >= u, u drawn from
//     Philox at counter (stream index, 3, epoch) -- every decision
//     reproducible;
//   - clusterisation: a candidate's neighbours are the older rods (all
//     periodic images) whose centres lie closer than half the longer length
//     to the candidate as drawn; they are visited in stream order, the
//     candidate moving after each snap; list building, a radix sort by
//     (candidate, rod, image) and one thread per candidate for the
//     sequential part.
#include <cmath>
#include <cstring>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "nf_engine.cuh"

namespace nf {

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

constexpr double kFix = 1099511627776.0;  // 2^40: resolution of the tensor sums

// ---------------------------------------------------------------------------
// Kernels.
// ---------------------------------------------------------------------------
// Per law cell: rod count and the six sums of c_i c_j in 2^-40 units.
__global__ void k_law_acc(uint32_t n, const Real* __restrict__ reals, const float4* __restrict__ pos,
                          const float4* __restrict__ dir, unsigned long long* __restrict__ acc) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Real& Re = reals[0];
    const float4 p = pos[i], c = dir[i];
    const uint32_t cell = law_cell(Re, p.x, p.y, p.z);
    const double x = c.x, y = c.y, z = c.z;
    const double pr[6] = {dmul(x, x), dmul(y, y), dmul(z, z), dmul(x, y), dmul(x, z), dmul(y, z)};
    unsigned long long* a = acc + 7 * (size_t)cell;
    atomicAdd(&a[0], 1ull);
#pragma unroll
    for (int k = 0; k < 6; ++k) atomicAdd(&a[1 + k], (unsigned long long)__double2ll_rn(dmul(pr[k], kFix)));
}

// Thin-out decisions: keep[i] = 1 when 2 F >= u (keep[n] = 0 for the scan).
__global__ void k_thin(uint32_t n, const Real* __restrict__ reals, const float4* __restrict__ pos,
                       const float4* __restrict__ dir, const uint64_t* __restrict__ sidx, uint32_t epoch,
                       uint32_t* __restrict__ keepf, uint32_t* __restrict__ removed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) { keepf[n] = 0u; return; }
    const Real& Re = reals[0];
    const float4 p = pos[i], c = dir[i];
    const float* Lw = Re.law + (size_t)kLawF * law_cell(Re, p.x, p.y, p.z);
    uint32_t k = 1u;
    if (Lw[9] > 0.0f) {
        const float d = fabsf(fadd(fadd(fmul(c.x, Lw[2]), fmul(c.y, Lw[5])), fmul(c.z, Lw[8])));
        const float F = exp_nf(fmul(Lw[9], fsub(d, 1.0f)));
        const uint64_t s = sidx[i];
        const U4 r = philox((uint32_t)s, (uint32_t)(s >> 32), 3u, epoch, Re.key[0], Re.key[1]);
        k = fmul(2.0f, F) >= uni(r.x) ? 1u : 0u;
    }
    keepf[i] = k;
    if (!k) atomicAdd(removed, 1u);
}

// Visits the older rods (index < n_old) of the candidate's stencil whose
// centres, over the periodic images -1..1, lie closer than half the longer
// length to the candidate: f(rod index, image code, rod).
template <class F>
__device__ __forceinline__ void clu_neighbours(const Real& Re, const float4& p, const uint32_t* __restrict__ rstart,
                                               const float4* __restrict__ spos, const uint32_t* __restrict__ sid,
                                               uint32_t n_old, F&& f) {
    int c0[3];
    const float v[3] = {p.x, p.y, p.z};
    for (int d = 0; d < 3; ++d) c0[d] = cell_coord(Re, d, v[d]);
    const int S = Re.S;
    for (int dz = -S; dz <= S; ++dz)
        for (int dy = -S; dy <= S; ++dy)
            for (int dx = -S; dx <= S; ++dx) {
                const int dd[3] = {dx, dy, dz};
                int cc[3], im[3];
                bool ok = true;
                for (int d = 0; d < 3 && ok; ++d) {
                    int q = c0[d] + dd[d];
                    im[d] = 0;
                    if (q < 0 || q >= Re.n[d]) {
                        if (!((Re.per_gen >> d) & 1)) { ok = false; break; }
                        im[d] = q < 0 ? -1 : 1;
                        q -= im[d] * Re.n[d];
                        if (q < 0 || q >= Re.n[d]) { ok = false; break; }  // beyond one image
                    }
                    cc[d] = q;
                }
                if (!ok) continue;
                const uint32_t cell = Re.cell_off + (uint32_t)(cc[0] + Re.n[0] * (cc[1] + Re.n[1] * cc[2]));
                const float sx = fmul((float)im[0], Re.L[0]), sy = fmul((float)im[1], Re.L[1]),
                            sz = fmul((float)im[2], Re.L[2]);
                const uint32_t code = (uint32_t)((im[0] + 1) + 3 * (im[1] + 1) + 9 * (im[2] + 1));
                for (uint32_t q = rstart[cell]; q < rstart[cell + 1]; ++q) {
                    const uint32_t j = sid[q];
                    if (j >= n_old) continue;
                    const float4 P = spos[q];
                    const float ex = fsub(fadd(P.x, sx), p.x), ey = fsub(fadd(P.y, sy), p.y),
                                ez = fsub(fadd(P.z, sz), p.z);
                    const float dist = fsqrt(fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez)));
                    if (dist < fmul(fmaxf(p.w, P.w), 0.5f)) f(j, code);
                }
            }
}

__global__ void k_clu_count(uint32_t slots, const uint32_t* __restrict__ ntot, const Real* __restrict__ reals,
                            const float4* __restrict__ cpos, const uint32_t* __restrict__ rstart,
                            const float4* __restrict__ spos, const uint32_t* __restrict__ sid, uint32_t n_old,
                            uint32_t* __restrict__ cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > slots) return;
    uint32_t k = 0;
    if (i < *ntot) clu_neighbours(reals[0], cpos[i], rstart, spos, sid, n_old, [&](uint32_t, uint32_t) { ++k; });
    cnt[i] = k;
}

__global__ void k_clu_fill(uint32_t i0, uint32_t i1, const Real* __restrict__ reals,
                           const float4* __restrict__ cpos, const uint32_t* __restrict__ rstart,
                           const float4* __restrict__ spos, const uint32_t* __restrict__ sid, uint32_t n_old,
                           const uint32_t* __restrict__ off, unsigned long long* __restrict__ key) {
    const uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    uint32_t w = off[i] - off[i0];
    clu_neighbours(reals[0], cpos[i], rstart, spos, sid, n_old, [&](uint32_t j, uint32_t code) {
        key[w++] = ((unsigned long long)i << 37) | ((unsigned long long)j << 5) | code;
    });
}

NF_HD float dot3f(float ax, float ay, float az, float bx, float by, float bz) {
    return fadd(fadd(fmul(ax, bx), fmul(ay, by)), fmul(az, bz));
}

// cnt_minDist (inc/intersection_dev.h:85-160) in FP32, each operation rounded
// on its own: the distance of the clamped closest points; *t0u, *t1u the
// parameters before the clamp (Dtt.y, Dtt.z). typo selects the reference's
// parallel branch (b.x in place of b.y and b.z, :122).
NF_HD float clu_min_dist(const float r1[3], const float c1[3], float l1, float a1, const float r2[3],
                         const float c2[3], float l2, float a2, float eps, bool typo, float* t0u, float* t1u) {
    const float bx = fsub(r2[0], r1[0]), by = fsub(r2[1], r1[1]), bz = fsub(r2[2], r1[2]);
    const float d = dot3f(c1[0], c1[1], c1[2], c2[0], c2[1], c2[2]);
    float t0, t1;
    if (fsub(1.0f, fabsf(d)) > eps) {
        float ax = fsub(fmul(d, c2[0]), c1[0]), ay = fsub(fmul(d, c2[1]), c1[1]), az = fsub(fmul(d, c2[2]), c1[2]);
        t0 = dot3f(ax, ay, az, bx, by, bz);
        ax = fsub(c2[0], fmul(d, c1[0]));
        ay = fsub(c2[1], fmul(d, c1[1]));
        az = fsub(c2[2], fmul(d, c1[2]));
        t1 = dot3f(ax, ay, az, bx, by, bz);
        const float den = fsub(fmul(d, d), 1.0f);
        t0 = fdiv(t0, den);
        t1 = fdiv(t1, den);
    } else {
        t0 = copysignf(fdiv(l1, 2.0f), dot3f(bx, by, bz, c1[0], c1[1], c1[2]));
        const float dt = typo ? fadd(fadd(fmul(bx, c2[0]), fmul(bx, c2[1])), fmul(bx, c2[2]))
                              : dot3f(bx, by, bz, c2[0], c2[1], c2[2]);
        t1 = fadd(fmul(-1.0f, dt), fmul(d, t0));
    }
    *t0u = t0;
    *t1u = t1;
    const float h1 = fdiv(l1, 2.0f), h2 = fdiv(l2, 2.0f);
    const bool f1 = fabsf(t0) <= fadd(fadd(h1, a1), eps);
    const bool f2 = fabsf(t1) <= fadd(fadd(h2, a2), eps);
    if (!(f1 && f2)) {
        const bool f3 = fsub(fabsf(t0), h1) < fsub(fabsf(t1), h2);
        if (f3) {  // the candidate's point follows from the rod's end
            t1 = copysignf(h2, t1);
            t0 = fadd(dot3f(bx, by, bz, c1[0], c1[1], c1[2]), fmul(d, t1));
            if (fabsf(t0) > h1) t0 = copysignf(h1, t0);
        } else {
            t0 = copysignf(h1, t0);
            t1 = fadd(fmul(-1.0f, dot3f(bx, by, bz, c2[0], c2[1], c2[2])), fmul(d, t0));
            if (fabsf(t1) > h2) t1 = copysignf(h2, t1);
        }
    }
    const float ex = fsub(fsub(fadd(r1[0], fmul(t0, c1[0])), r2[0]), fmul(t1, c2[0]));
    const float ey = fsub(fsub(fadd(r1[1], fmul(t0, c1[1])), r2[1]), fmul(t1, c2[1]));
    const float ez = fsub(fsub(fadd(r1[2], fmul(t0, c1[2])), r2[2]), fmul(t1, c2[2]));
    return fsqrt(fadd(fadd(fmul(ex, ex), fmul(ey, ey)), fmul(ez, ez)));
}

// The sequential part: one thread per kept candidate walks its neighbours in
// (rod, image) order and snaps; then the centre is wrapped on periodic axes,
// and a candidate left outside the box on an open axis is rejected. Cell of
// the final centre recounted for the binning.
__global__ void k_clu_apply(uint32_t i0, uint32_t i1, const Real* __restrict__ reals,
                            const uint32_t* __restrict__ off, const unsigned long long* __restrict__ key,
                            const float4* __restrict__ pos, const float4* __restrict__ dir, float cos_lim,
                            float dist_lim, float4* __restrict__ cpos, float4* __restrict__ cdir,
                            uint8_t* __restrict__ state, uint32_t* __restrict__ ccell, uint32_t* __restrict__ ccount,
                            uint32_t* __restrict__ nsnap) {
    const uint32_t i = i0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= i1) return;
    const Real& Re = reals[0];
    float4 P = cpos[i], C = cdir[i];
    float r1[3] = {P.x, P.y, P.z}, c1[3] = {C.x, C.y, C.z};
    const float l1 = P.w, a1 = C.w;
    unsigned snaps = 0;
    for (uint32_t e = off[i] - off[i0]; e < off[i + 1] - off[i0]; ++e) {
        const unsigned long long kk = key[e];
        const uint32_t j = (uint32_t)((kk >> 5) & 0xffffffffull), code = (uint32_t)(kk & 31ull);
        const int im[3] = {(int)(code % 3) - 1, (int)((code / 3) % 3) - 1, (int)(code / 9) - 1};
        const float4 Q = pos[j], D = dir[j];
        const float r2[3] = {fadd(Q.x, fmul((float)im[0], Re.L[0])), fadd(Q.y, fmul((float)im[1], Re.L[1])),
                             fadd(Q.z, fmul((float)im[2], Re.L[2]))};
        const float c2[3] = {D.x, D.y, D.z};
        const float ex = fsub(r1[0], r2[0]), ey = fsub(r1[1], r2[1]), ez = fsub(r1[2], r2[2]);
        if (!(fsqrt(dot3f(ex, ey, ez, ex, ey, ez)) < fmul(fmaxf(l1, Q.w), 0.5f))) continue;
        if (!(fabsf(dot3f(c1[0], c1[1], c1[2], c2[0], c2[1], c2[2])) >= cos_lim)) continue;
        float t0, t1;
        const float d = clu_min_dist(r1, c1, l1, a1, r2, c2, Q.w, D.w, Re.eps, Re.typo != 0, &t0, &t1);
        if (!(d <= dist_lim)) continue;
        // cuda_Clusterize2Old, inc/cuda_Clusterize.h:81-88
        float vx = fsub(fadd(r1[0], fmul(c1[0], t0)), fadd(r2[0], fmul(c2[0], t1)));
        float vy = fsub(fadd(r1[1], fmul(c1[1], t0)), fadd(r2[1], fmul(c2[1], t1)));
        float vz = fsub(fadd(r1[2], fmul(c1[2], t0)), fadd(r2[2], fmul(c2[2], t1)));
        const float vc = dot3f(vx, vy, vz, c2[0], c2[1], c2[2]);
        vx = fsub(vx, fmul(c2[0], vc));
        vy = fsub(vy, fmul(c2[1], vc));
        vz = fsub(vz, fmul(c2[2], vc));
        const float nv = fsqrt(dot3f(vx, vy, vz, vx, vy, vz));
        if (!(nv > 0.0f)) continue;  // axes meet: no direction to move along
        const float inv = fdiv(1.0f, nv);
        vx = fmul(vx, inv);
        vy = fmul(vy, inv);
        vz = fmul(vz, inv);
        const float sd = fadd(fadd(a1, D.w), Re.sep);
        const float tt = fmul(dot3f(c1[0], c1[1], c1[2], c2[0], c2[1], c2[2]), t0);
        const float q[3] = {fadd(r2[0], fmul(c2[0], t1)), fadd(r2[1], fmul(c2[1], t1)), fadd(r2[2], fmul(c2[2], t1))};
        r1[0] = fsub(fadd(q[0], fmul(vx, sd)), fmul(c2[0], tt));
        r1[1] = fsub(fadd(q[1], fmul(vy, sd)), fmul(c2[1], tt));
        r1[2] = fsub(fadd(q[2], fmul(vz, sd)), fmul(c2[2], tt));
        c1[0] = c2[0];
        c1[1] = c2[1];
        c1[2] = c2[2];
        ++snaps;
    }
    bool inside = true;
    for (int d = 0; d < 3; ++d) {
        if ((Re.per_gen >> d) & 1) {
            if (r1[d] < 0.0f) r1[d] = fadd(r1[d], Re.L[d]);
            if (r1[d] >= Re.L[d]) r1[d] = fsub(r1[d], Re.L[d]);
        }
        if (!(r1[d] >= 0.0f && r1[d] < Re.L[d])) inside = false;
    }
    if (snaps) {
        cpos[i] = make_float4(r1[0], r1[1], r1[2], l1);
        cdir[i] = make_float4(c1[0], c1[1], c1[2], a1);
    }
    nsnap[i] = snaps;
    if (!inside) state[i] = ST_REJ_OLD;
    const uint32_t cell = cell_of(Re, r1[0], r1[1], r1[2]);
    ccell[i] = cell;
    atomicAdd(&ccount[cell], 1u);
}

// Snaps of the round's candidates with stream index below the round's stop.
__global__ void k_snap_sum(uint32_t slots, const uint32_t* __restrict__ ntot, const uint64_t* __restrict__ csidx,
                           uint64_t limit, const uint32_t* __restrict__ nsnap, unsigned long long* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= slots || i >= *ntot || csidx[i] >= limit || !nsnap[i]) return;
    atomicAdd(out, (unsigned long long)nsnap[i]);
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
bool Engine::adaptive() const { return R == 1 && (prm[0].self_align_step > 0 || prm[0].clust_flag); }

// Law grid of a realisation: cells of edge >= align_cell (the rod length when
// 0) per axis.
static void law_grid(const nf_params& p, int32_t n[3], float inv[3]) {
    const double e = p.align_cell > 0 ? (double)p.align_cell : (double)p.l;
    for (int d = 0; d < 3; ++d) {
        const double c = std::floor((double)p.box[d] / e);
        n[d] = c < 1 ? 1 : (c > 256 ? 256 : (int32_t)c);
        inv[d] = (float)((double)n[d] / (double)p.box[d]);
    }
}

// The global law of the realisation in the law layout.
static void global_law(const Real& Re, float* Lw) {
    for (int k = 0; k < 9; ++k) Lw[k] = Re.m[k];
    Lw[9] = Re.orient == 1 ? Re.kappa : 0.0f;
    Lw[10] = Re.orient == 1 ? Re.E2 : 0.0f;
    Lw[11] = (float)((Re.orient == 1 ? 1 : 0) | (Re.rot ? 2 : 0));
    Lw[12] = 0.0f;
    Lw[13] = 0.0f;
}

nf_status Engine::laws_reset() {
    if (!adaptive()) {
        hreal[0].law = nullptr;
        laws_set = false;
        return NF_OK;
    }
    float inv[3];
    law_grid(prm[0], lawn, inv);
    const size_t nc = (size_t)lawn[0] * lawn[1] * lawn[2];
    hlaw.assign(nc * kLawF, 0.0f);
    for (size_t c = 0; c < nc; ++c) global_law(hreal[0], &hlaw[c * kLawF]);
    hlawd.assign(nc * kLawD, 0.0);
    NF_CK(law.ensure(nc * kLawF));
    NF_CK(lawd.ensure(nc * kLawD));
    NF_CK(lacc.ensure(nc * 7));
    NF_CK(cudaMemcpyAsync(law.p, hlaw.data(), sizeof(float) * hlaw.size(), cudaMemcpyHostToDevice, st));
    NF_CK(cudaMemcpyAsync(lawd.p, hlawd.data(), sizeof(double) * hlawd.size(), cudaMemcpyHostToDevice, st));
    Real& Re = hreal[0];
    Re.law = law.p;
    Re.lawd = lawd.p;
    for (int d = 0; d < 3; ++d) {
        Re.an[d] = lawn[d];
        Re.ainv[d] = inv[d];
    }
    NF_CK(cudaMemcpyAsync(dreal.p, &Re, sizeof(Real), cudaMemcpyHostToDevice, st));
    laws_set = true;
    return NF_OK;
}

// Cyclic Jacobi on a symmetric 3x3 matrix (FP64): A becomes diagonal, V holds
// the eigenvectors in its columns.
static void jacobi3(double A[3][3], double V[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) V[i][j] = i == j ? 1.0 : 0.0;
    static const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 64; ++sweep) {
        if (A[0][1] == 0.0 && A[0][2] == 0.0 && A[1][2] == 0.0) break;
        for (const auto& pq : P) {
            const int p = pq[0], q = pq[1];
            if (A[p][q] == 0.0) continue;
            const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
            const double at = th < 0 ? -th : th;
            double t = at > 1e150 ? 0.5 / at : 1.0 / (at + std::sqrt(th * th + 1.0));
            if (th < 0) t = -t;
            const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
            for (int k = 0; k < 3; ++k) {  // A <- A J
                const double akp = A[k][p], akq = A[k][q];
                A[k][p] = c * akp - s * akq;
                A[k][q] = s * akp + c * akq;
            }
            for (int k = 0; k < 3; ++k) {  // A <- J^T A
                const double apk = A[p][k], aqk = A[q][k];
                A[p][k] = c * apk - s * aqk;
                A[q][k] = s * apk + c * aqk;
            }
            A[p][q] = A[q][p] = 0.0;
            for (int k = 0; k < 3; ++k) {  // V <- V J
                const double vkp = V[k][p], vkq = V[k][q];
                V[k][p] = c * vkp - s * vkq;
                V[k][q] = s * vkp + c * vkq;
            }
        }
    }
}

// Second moment E[(c.mu)^2] of the von Mises-Fisher law of concentration k.
static double vmf_m2(double k) {
    if (k < 0.05) {
        const double k2 = k * k;
        return 1.0 / 3.0 + k2 * (2.0 / 45.0 - k2 * (4.0 / 945.0));
    }
    return 1.0 - 2.0 / (k * std::tanh(k)) + 2.0 / (k * k);
}

// The law of a cell from its sums (count, xx, yy, zz, xy, xz, yz). The
// candidates draw from it only when the realisation's own law has a spread
// (von Mises-Fisher): the reference samples isotropically whatever the cell
// laws while DEF_THETA_DEV is -1 (genCosine, inc/cuda_CNTgenerate.h:262-270);
// thin-out uses the fitted law in either case.
static void fit_law(const long long s[7], bool sample, float* Lw) {
    const double n = (double)s[0];
    double A[3][3];
    const double f = 1.0 / (n * kFix);
    A[0][0] = (double)s[1] * f;
    A[1][1] = (double)s[2] * f;
    A[2][2] = (double)s[3] * f;
    A[0][1] = A[1][0] = (double)s[4] * f;
    A[0][2] = A[2][0] = (double)s[5] * f;
    A[1][2] = A[2][1] = (double)s[6] * f;
    double V[3][3];
    jacobi3(A, V);
    int b = 0;
    for (int k = 1; k < 3; ++k)
        if (A[k][k] > A[b][b]) b = k;
    double mu[3] = {V[0][b], V[1][b], V[2][b]};
    const double nm = std::sqrt(mu[0] * mu[0] + mu[1] * mu[1] + mu[2] * mu[2]);
    for (double& v : mu) v /= nm;
    // axes are unsigned: the sign with mu_z > 0 (then mu_y, then mu_x)
    const bool flip = mu[2] < 0 || (mu[2] == 0 && (mu[1] < 0 || (mu[1] == 0 && mu[0] < 0)));
    if (flip)
        for (double& v : mu) v = -v;
    const double lam = A[b][b];
    double kappa = 0.0;
    if (lam > 1.0 / 3.0 + 1e-9) {
        double lo = 0.0, hi = 500.0;
        if (vmf_m2(hi) <= lam) {
            kappa = hi;
        } else {
            for (int it = 0; it < 64; ++it) {
                const double mid = 0.5 * (lo + hi);
                if (vmf_m2(mid) < lam) lo = mid; else hi = mid;
            }
            kappa = 0.5 * (lo + hi);
        }
    }
    // rotation taking z to mu: the orthonormal basis of Duff et al. (2017),
    // "Building an Orthonormal Basis, Revisited", in its columns t1, t2, mu
    const double sg = mu[2] >= 0 ? 1.0 : -1.0;
    const double a = -1.0 / (sg + mu[2]), bb = mu[0] * mu[1] * a;
    const double t1[3] = {1.0 + sg * mu[0] * mu[0] * a, sg * bb, -sg * mu[0]};
    const double t2[3] = {bb, sg + mu[1] * mu[1] * a, -mu[1]};
    for (int r = 0; r < 3; ++r) {
        Lw[3 * r + 0] = (float)t1[r];
        Lw[3 * r + 1] = (float)t2[r];
        Lw[3 * r + 2] = (float)mu[r];
    }
    const float kf = (float)kappa;
    Lw[9] = kf;
    Lw[10] = (float)std::exp(-2.0 * (double)kf);
    Lw[11] = sample ? (float)((kf > 0.0f ? 1 : 0) | 2) : 0.0f;
}

// ALIGN_LAW 1: the reference's cell law (crossMtxBuild, resetOrt,
// resetAvgVec; inc/allignment_fit.h:154-210, 214-274, 353-458), fitted on the
// host in FP64 from the cell's rods in rod order:
//   - preferred axis: the unit eigenvector of <c c^T> of the largest
//     eigenvalue when the two smaller eigenvalues (by magnitude) are within
//     10 % of each other ("cone-like"), else of the smallest ("disk-like"),
//     signed with v_z > 0 (then v_y, v_x); theta_o = acos(v_z),
//     phi_o = acos(v_x / sin theta_o) with the reference's 1e-6 guards; the
//     draw is rotated by inc_rotation(Mu = phi_o, Xi = -theta_o);
//   - law: when the mean of the rods' directions has a norm per rod above
//     0.5 (def_minOrtNorm, src/simPrms.cpp:42), theta = asin |a_xy|,
//     phi = acos(a_x / |a_xy|) of the unit mean a, and the mean squared
//     deviations of asin |c_xy| and acos(c_x / |c_xy|) from them are the
//     scales of the truncated-normal draws (the reference hands its "mean
//     squared deviation" arrays to sym_truncNormal as s). The angles are taken
//     in the box frame: the reference's rotation into the preferred frame
//     (rot_Z / rot_Y on a float3, whose result is discarded) leaves the
//     vectors as they are. Otherwise the cell keeps its truncated-normal laws.
// Angles of a direction in the box frame (Ort2Angle, inc/vectorMath.h:85-90).
static void box_angles(double cx, double cy, double* th, double* ph) {
    const double nxy = std::sqrt(cx * cx + cy * cy);
    *th = std::asin(nxy > 1.0 ? 1.0 : nxy);
    double q = nxy > 1e-6 ? cx / nxy : 0.0;
    q = q > 1.0 ? 1.0 : (q < -1.0 ? -1.0 : q);
    *ph = nxy > 1e-6 ? std::acos(q) : 0.0;
}

static void fit_tn_cell(const float4* dirs, const std::vector<uint32_t>& idx, int ref, float* Lw, double* Ld) {
    const double n = (double)idx.size();
    double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double ax = 0, ay = 0, az = 0;
    for (uint32_t i : idx) {
        const double x = dirs[i].x, y = dirs[i].y, z = dirs[i].z;
        A[0][0] += x * x; A[1][1] += y * y; A[2][2] += z * z;
        A[0][1] += x * y; A[0][2] += x * z; A[1][2] += y * z;
        ax += x; ay += y; az += z;
    }
    for (int r = 0; r < 3; ++r)
        for (int c = r; c < 3; ++c) A[r][c] /= n;
    A[1][0] = A[0][1]; A[2][0] = A[0][2]; A[2][1] = A[1][2];
    double V[3][3];
    jacobi3(A, V);
    int o[3] = {0, 1, 2};  // eigenvalues by decreasing magnitude
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b)
            if (std::fabs(A[o[b]][o[b]]) > std::fabs(A[o[a]][o[a]])) std::swap(o[a], o[b]);
    const double e1 = A[o[1]][o[1]], e2 = A[o[2]][o[2]];
    const int k = std::fabs((e1 - e2) / e1) < 0.1 ? o[0] : o[2];
    double v[3] = {V[0][k], V[1][k], V[2][k]};
    const double nv = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (double& q : v) q /= nv;
    if (v[2] < 0 || (v[2] == 0 && (v[1] < 0 || (v[1] == 0 && v[0] < 0))))
        for (double& q : v) q = -q;
    const double tho = std::fabs(v[2]) <= 1.0 - 1e-6 ? std::acos(v[2]) : (v[2] > 0 ? 0.0 : kPiD);
    const double sth = std::sin(tho);
    double cph = std::fabs(sth) > 1e-6 ? v[0] / sth : 1.0;
    const double pho = std::fabs(cph) <= 1.0 - 1e-6 ? std::acos(cph) : (cph > 0 ? 0.0 : kPiD);
    float cM, sM, cX, sX;  // inc_rotation, Mu = phi_o, Xi = -theta_o (as the global PREF_ORT rotation)
    sincos_turns((float)(pho / (2.0 * kPiD)), &cM, &sM);
    sincos_turns((float)(-tho / (2.0 * kPiD)), &cX, &sX);
    Lw[0] = fmul(cM, cX);  Lw[1] = sM;   Lw[2] = fmul(-sX, cM);
    Lw[3] = fmul(-sM, cX); Lw[4] = cM;   Lw[5] = fmul(sX, sM);
    Lw[6] = sX;            Lw[7] = 0.0f; Lw[8] = cX;
    Lw[9] = 0.0f;
    Lw[10] = 0.0f;
    int fl = 2 | ((int)Lw[11] & 4);
    const double na = std::sqrt(ax * ax + ay * ay + az * az);
    if (na / n > 0.5) {
        double th, ph;
        box_angles(ax / na, ay / na, &th, &ph);
        double st = 0.0, sp = 0.0;
        for (uint32_t i : idx) {
            double dt, dp;
            box_angles(dirs[i].x, dirs[i].y, &dt, &dp);
            st += (dt - th) * (dt - th);
            sp += (dp - ph) * (dp - ph);
        }
        // the reference keeps these in float arrays; a zero spread is kept
        // finite (all of the cell's rods parallel: the draws collapse onto the mean)
        const float ft = (float)th, fp = (float)ph;
        const float dt = std::max((float)(st / n), 1e-12f), dp = std::max((float)(sp / n), 1e-12f);
        Lw[12] = ft;
        Lw[13] = fp;
        Ld[0] = ft; Ld[1] = dt; Ld[2] = fp; Ld[3] = dp;
        tn_consts(dt, kPiD * 0.5, ref, &Ld[4], &Ld[5], &Ld[6]);
        tn_consts(dp, kPiD, ref, &Ld[7], &Ld[8], &Ld[9]);
        fl |= 4;
    }
    Lw[11] = (float)fl;
}

// Thin-out under ALIGN_LAW 1 (randomThinOut / check_probability,
// inc/allignment_fit.h:466-578): F = exp(-((theta - theta_m) / s_theta)^2 / 2)
// exp(-((phi - phi_m) / s_phi)^2 / 2) in the box frame, a factor 1 where a
// scale is 0; the rod stays when 2 F >= u, u from Philox at (stream index, 3,
// epoch). Rods of cells without a fitted law stay.
static bool tn_keep(const Real& Re, const float* Lw, const double* Ld, const float4& c, uint64_t si, uint32_t epoch) {
    if (!(((int)Lw[11]) & 4)) return true;
    double th, ph;
    box_angles(c.x, c.y, &th, &ph);
    const double qt = (th - Ld[0]) / Ld[1], qp = (ph - Ld[2]) / Ld[3];
    const double F = std::exp(-0.5 * qt * qt) * std::exp(-0.5 * qp * qp);
    const U4 r = philox((uint32_t)si, (uint32_t)(si >> 32), 3u, epoch, Re.key[0], Re.key[1]);
    return 2.0 * F >= (double)uni(r.x);
}

nf_status Engine::epoch_boundary(uint64_t e, uint32_t gained) {
    const nf_params& p = prm[0];
    const uint32_t n = count[0];
    const uint32_t tgt = hreal[0].target;
    const int s = p.self_align_step;
    const bool refit = s > 0 && e > 0 && ((e % (uint64_t)s) == 0 || (double)gained < (double)(tgt - n) / 100.0);
    if (!refit) return NF_OK;
    const size_t nc = (size_t)lawn[0] * lawn[1] * lawn[2];
    if (p.align_law == 1) return epoch_boundary_tn(e, n);
    NF_CK(cudaMemsetAsync(lacc.p, 0, sizeof(unsigned long long) * 7 * nc, st));
    if (n) NF_LAUNCH(k_law_acc, grid_for(n, 256), 256, 0, st)(n, dreal.p, pos.p, dir.p, lacc.p);
    NF_CK(cudaGetLastError());
    std::vector<long long> hs(7 * nc);
    NF_CK(cudaMemcpyAsync(hs.data(), lacc.p, sizeof(long long) * 7 * nc, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    const long long need = p.align_min > 0 ? p.align_min : 1;
    for (size_t c = 0; c < nc; ++c)
        if (hs[7 * c] >= need) fit_law(&hs[7 * c], p.orient_mode == NF_ORIENT_VMF, &hlaw[c * kLawF]);
    NF_CK(cudaMemcpyAsync(law.p, hlaw.data(), sizeof(float) * hlaw.size(), cudaMemcpyHostToDevice, st));
    ++ad_refits;
    if (p.reduce_flag && n) {
        DBuf<uint32_t> kf, rm;
        NF_CK(kf.ensure(n + 1));
        NF_CK(rm.ensure(1));
        NF_CK(cudaMemsetAsync(rm.p, 0, sizeof(uint32_t), st));
        NF_LAUNCH(k_thin, grid_for(n + 1, 256), 256, 0, st)(n, dreal.p, pos.p, dir.p, sidx.p, (uint32_t)(e + 1), kf.p,
                                                          rm.p);
        NF_CK(cudaGetLastError());
        uint32_t removed = 0;
        NF_CK(cudaMemcpyAsync(&removed, rm.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        if (removed) {
            nf_status r = compact_rods(kf.p, n, n - removed);
            if (r != NF_OK) return r;
            ad_thinned += removed;
        }
    }
    return NF_OK;
}

// Refit (and thin-out) under ALIGN_LAW 1 after epoch e: the rods come to the
// host, the cell laws are fitted there in FP64 (fit_tn_cell) and the thin-out
// decided there (tn_keep).
nf_status Engine::epoch_boundary_tn(uint64_t e, uint32_t n) {
    const nf_params& p = prm[0];
    const size_t nc = (size_t)lawn[0] * lawn[1] * lawn[2];
    std::vector<float4> hp(n), hd(n);
    std::vector<uint64_t> hs(n);
    if (n) {
        NF_CK(cudaMemcpyAsync(hp.data(), pos.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(hd.data(), dir.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(hs.data(), sidx.p, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
    }
    const Real& Re = hreal[0];
    std::vector<std::vector<uint32_t>> members(nc);
    for (uint32_t i = 0; i < n; ++i) members[law_cell(Re, hp[i].x, hp[i].y, hp[i].z)].push_back(i);
    const size_t need = p.align_min > 0 ? (size_t)p.align_min : 1;
    for (size_t c = 0; c < nc; ++c)
        if (members[c].size() >= need)
            fit_tn_cell(hd.data(), members[c], p.ref_trunc_normal, &hlaw[c * kLawF], &hlawd[c * kLawD]);
    NF_CK(cudaMemcpyAsync(law.p, hlaw.data(), sizeof(float) * hlaw.size(), cudaMemcpyHostToDevice, st));
    NF_CK(cudaMemcpyAsync(lawd.p, hlawd.data(), sizeof(double) * hlawd.size(), cudaMemcpyHostToDevice, st));
    ++ad_refits;
    if (!(p.reduce_flag && n)) return NF_OK;
    std::vector<uint32_t> keepf(n + 1, 0u);
    uint32_t removed = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const size_t c = law_cell(Re, hp[i].x, hp[i].y, hp[i].z);
        keepf[i] = tn_keep(Re, &hlaw[c * kLawF], &hlawd[c * kLawD], hd[i], hs[i], (uint32_t)(e + 1)) ? 1u : 0u;
        removed += keepf[i] ? 0u : 1u;
    }
    if (!removed) return NF_OK;
    DBuf<uint32_t> kf;
    NF_CK(kf.ensure(n + 1));
    NF_CK(cudaMemcpyAsync(kf.p, keepf.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, st));
    nf_status r = compact_rods(kf.p, n, n - removed);
    if (r != NF_OK) return r;
    ad_thinned += removed;
    return NF_OK;
}

// Neighbour keys held at once: the round's candidates are processed in chunks
// whose lists fit (2 x 1 GB of keys), so a dense box with many candidates
// per round does not need one list for all of them.
constexpr uint64_t kCluKeyCap = 1ull << 27;

nf_status Engine::clusterize(uint64_t slots, const uint32_t* ntot, uint32_t n_old) {
    const nf_params& p = prm[0];
    NF_CK(clu_cnt.ensure(slots + 1));
    NF_CK(clu_off.ensure(slots + 1));
    NF_CK(clu_snaps.ensure(slots + 1));
    const unsigned gs = grid_for(slots + 1, 256);
    NF_LAUNCH(k_clu_count, gs, 256, 0, st)((uint32_t)slots, ntot, dreal.p, cpos.p, rstart.p, spos.p, sid.p, n_old,
                                           clu_cnt.p);
    NF_CK(cudaGetLastError());
    nf_status s = scan_u32(clu_cnt.p, clu_off.p, slots + 1);
    if (s != NF_OK) return s;
    uint32_t hn = 0, total = 0;
    NF_CK(cudaMemcpyAsync(&hn, ntot, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaMemcpyAsync(&total, clu_off.p + slots, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    // chunks of candidates [i0, i1) with at most kCluKeyCap keys each
    std::vector<uint32_t> cuts{0u};
    if ((uint64_t)total > kCluKeyCap) {
        std::vector<uint32_t> ho(hn + 1);
        NF_CK(cudaMemcpyAsync(ho.data(), clu_off.p, sizeof(uint32_t) * (hn + 1), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        uint32_t i0 = 0;
        while (i0 < hn) {
            uint32_t i1 = i0 + 1;
            while (i1 < hn && (uint64_t)ho[i1 + 1] - ho[i0] <= kCluKeyCap) ++i1;
            cuts.push_back(i1);
            i0 = i1;
        }
    } else {
        cuts.push_back(hn);
    }
    const uint64_t cap = std::min<uint64_t>(total, kCluKeyCap) + 1;
    NF_CK(clu_key.ensure(cap));
    NF_CK(clu_key2.ensure(cap));
    // the snap moves centres: recount the cells
    NF_CK(cudaMemsetAsync(ccount.p, 0, sizeof(uint32_t) * (ncell + 1), st));
    const float cos_lim = (float)std::cos((double)p.clust_angl);
    for (size_t c = 0; c + 1 < cuts.size(); ++c) {
        const uint32_t i0 = cuts[c], i1 = cuts[c + 1];
        if (i1 <= i0) continue;
        const unsigned gc = grid_for(i1 - i0, 256);
        NF_LAUNCH(k_clu_fill, gc, 256, 0, st)(i0, i1, dreal.p, cpos.p, rstart.p, spos.p, sid.p, n_old, clu_off.p,
                                              clu_key.p);
        NF_CK(cudaGetLastError());
        uint32_t nk = 0;
        NF_CK(cudaMemcpyAsync(&nk, clu_off.p + i1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        uint32_t nk0 = 0;
        NF_CK(cudaMemcpyAsync(&nk0, clu_off.p + i0, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        nk -= nk0;
        if (nk) {
            g_launches += 1;
            size_t bytes = 0;
            NF_CK(cub::DeviceRadixSort::SortKeys(nullptr, bytes, clu_key.p, clu_key2.p, (int)nk, 0, 61, st));
            NF_CK(cubtmp.ensure(bytes));
            NF_CK(cub::DeviceRadixSort::SortKeys(cubtmp.p, bytes, clu_key.p, clu_key2.p, (int)nk, 0, 61, st));
        }
        NF_LAUNCH(k_clu_apply, gc, 256, 0, st)(i0, i1, dreal.p, clu_off.p, clu_key2.p, pos.p, dir.p, cos_lim,
                                               p.clust_dist, cpos.p, cdir.p, state.p, ccell.p, ccount.p, clu_snaps.p);
        NF_CK(cudaGetLastError());
    }
    return NF_OK;
}

nf_status Engine::count_snaps(uint64_t slots, const uint32_t* ntot, uint64_t limit) {
    DBuf<unsigned long long> ns;
    NF_CK(ns.ensure(1));
    NF_CK(cudaMemsetAsync(ns.p, 0, sizeof(unsigned long long), st));
    NF_LAUNCH(k_snap_sum, grid_for(slots + 1, 256), 256, 0, st)((uint32_t)slots, ntot, csidx.p, limit, clu_snaps.p, ns.p);
    NF_CK(cudaGetLastError());
    unsigned long long hn = 0;
    NF_CK(cudaMemcpyAsync(&hn, ns.p, sizeof(hn), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    ad_snapped += hn;
    return NF_OK;
}

nf_status Engine::orientation_laws(size_t cap, int32_t ext[3], float* axis, float* kappa, size_t* cells) {
    if (!laws_set) { err = "the handle generates without adaptive orientation laws"; return NF_ERR_STATE; }
    const size_t nc = (size_t)lawn[0] * lawn[1] * lawn[2];
    if (cells) *cells = nc;
    if (ext) for (int d = 0; d < 3; ++d) ext[d] = lawn[d];
    if ((axis || kappa) && cap < nc) { err = "law buffers too small"; return NF_ERR_CAPACITY; }
    for (size_t c = 0; c < nc; ++c) {
        const float* Lw = &hlaw[c * kLawF];
        if (axis) {
            axis[3 * c + 0] = Lw[2];
            axis[3 * c + 1] = Lw[5];
            axis[3 * c + 2] = Lw[8];
        }
        if (kappa) kappa[c] = Lw[9];
    }
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
