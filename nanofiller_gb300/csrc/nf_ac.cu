// nf_ac.cu -- AC admittance spectrum of the conductance network: the offline
// Kirchhoff tool's impedance sweep (tools/kirchhoff/kirchhoff.py:55-286),
// restated for the GPU.
//
// Edge admittances (scaled by R0, the tool's unit):
//   rod segment   G = sigma pi a / L * R0, C = 0            (kirchhoff.py:90-95)
//   contact       d = max(D - 2 r_cnt, delta_min), S clamped to [S_min, S_max],
//                 kept only if d < delta_eff                 (kirchhoff.py:141-172)
//                 G = 1 / (exp(B (d - delta_min)) (d / delta_min) / (S / S_min))
//                     if d <= delta_tun, else 0             (kirchhoff.py:106-116)
//                 C = (S / S_min) / (d / delta_min), 0 below c_min
//                                                            (kirchhoff.py:97-104)
// At frequency f the admittance is Y = G + i (2 pi f / omega0) C; the system
// diag(sum of Y at the node) - A - A^T (complex symmetric) with the source at
// 1 and the sink at 0 in Norton form (kirchhoff.py:232-238); I = sum over the
// source contacts of Y_src (1 - V) (kirchhoff.py:266).
//
// GB300 form: the active-set CSR holds (G, C) pairs once; every frequency of a
// call is one CTA of one launch, which forms its own admittances on the fly,
// factors its own complex chain preconditioner (the tridiagonal rod chains of
// the intra-rod network; Jacobi elsewhere) and runs COCG (conjugate
// orthogonal CG, the CG of complex-symmetric systems: bilinear r^T z, no
// conjugation) in FP64, restarted from the true residual. FP64 because the
// tool's laws put admittances 1e11-1e12 apart in one network (a rod segment
// ~5e4 R0^-1, a contact at the tunnelling range ~1e-7), which FP32 vectors
// cannot resolve (2^-24 ~ 6e-8 of the largest term). Pivots of a chain are
// series combinations of admittances with G, C >= 0, so they stay in the
// first quadrant and no cancellation arises.
#include <algorithm>
#include <cmath>
#include <vector>

#include "nf_engine.cuh"
#include "nf_graph.cuh"

namespace nf {

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

// Physical constants (CODATA 2022; kirchhoff.py takes them from scipy.constants).
constexpr double kMe = 9.1093837139e-31;     // kg
constexpr double kH = 6.62607015e-34;        // J s
constexpr double kE = 1.602176634e-19;       // C
constexpr double kEps0 = 8.8541878188e-12;   // F / m
constexpr double kPi = 3.141592653589793;

struct AcConst {
    double dmin, dtun, deff, smin, smax, B, cmin, r2;  // SI units; r2 = 2 r_cnt (m)
    int own_radii;
};

// Contact admittance (scaled G, C). D in um, S in um^2; ra, rb: the rods'
// radii in um when own_radii (rb = 0 for an electrode contact). Every
// operation is rounded on its own (no contraction into FMA), so the kernels
// that inline this agree bit for bit, and with a plain FP64 evaluation.
__device__ __forceinline__ void ac_contact(const AcConst& k, double D, double S, double ra, double rb, double* G,
                                           double* C) {
    double d = k.own_radii ? dsub(dmul(D, 1e-6), dmul(dadd(ra, rb), 1e-6)) : dsub(dmul(D, 1e-6), k.r2);
    d = d > k.dmin ? d : k.dmin;
    double s = dmul(S, 1e-12);
    s = s > k.smin ? s : k.smin;
    s = s <= k.smax ? s : k.smax;
    if (!(d < k.deff)) { *G = 0.0; *C = 0.0; return; }
    const double sr = ddiv(s, k.smin), dr = ddiv(d, k.dmin);
    *G = d <= k.dtun ? ddiv(1.0, ddiv(dmul(exp(dmul(k.B, dsub(d, k.dmin))), dr), sr)) : 0.0;
    const double c = ddiv(sr, dr);
    *C = c < k.cmin ? 0.0 : c;
}

// Contacts of the handle's network: edge e joins rod I[e] to rod J[e] (or an
// electrode); radii from the rods' direction records.
__global__ void k_ac_contacts(uint32_t m, const uint32_t* __restrict__ rodI, const uint32_t* __restrict__ rodJ,
                              const double* __restrict__ D, const double* __restrict__ S,
                              const float4* __restrict__ dir, AcConst k, double* __restrict__ G,
                              double* __restrict__ C) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    double ra = 0.0, rb = 0.0;
    if (k.own_radii) {
        ra = (double)dir[rodI[e]].w;
        const uint32_t j = rodJ[e];
        rb = j < NF_SNK_ELEC ? (double)dir[j].w : 0.0;
    }
    ac_contact(k, D[e], S[e], ra, rb, &G[e], &C[e]);
}

// Contacts of a host-given network (the tool's radius convention only).
__global__ void k_ac_contacts_net(uint32_t m, const double* __restrict__ D, const double* __restrict__ S, AcConst k,
                                  double* __restrict__ G, double* __restrict__ C) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    ac_contact(k, D[e], S[e], 0.0, 0.0, &G[e], &C[e]);
}

// Segments from their DC conductance (sigma pi a / L, in S): scaled by R0.
__global__ void k_ac_segs_g(uint32_t ns, const double* __restrict__ g, double R0, double* __restrict__ G,
                            double* __restrict__ C) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    G[s] = dmul(g[s], R0);
    C[s] = 0.0;
}

// Segments of a host-given network: the same law from (L, a).
__global__ void k_ac_segs_la(uint32_t ns, const double* __restrict__ L, const double* __restrict__ a, double sigma,
                             double R0, double* __restrict__ G, double* __restrict__ C) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    G[s] = dmul(ddiv(dmul(dmul(sigma, kPi), a[s]), L[s]), R0);  // as the intra-rod network forms it, times R0
    C[s] = 0.0;
}

// Union-find kernels of the network assembly (nf_solve.cu).
__global__ void k_uf_init(uint32_t n, uint32_t* parent, uint32_t* flag);
__global__ void k_uf_union(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                           const double* __restrict__ G, const double* __restrict__ C, uint32_t* parent,
                           uint32_t* err);
__global__ void k_uf_flags(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                           const double* __restrict__ G, const double* __restrict__ C, uint32_t* parent,
                           uint32_t* flag, uint32_t* err);

__global__ void k_ac_chi(uint32_t n, const uint32_t* __restrict__ act, const uint32_t* __restrict__ aidx,
                         uint32_t* parent, const uint32_t* __restrict__ flag, double* __restrict__ chi, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !act[i]) return;
    chi[aidx[i]] = (flag[uf_find(parent, i, err)] & 1u) ? 1.0 : 0.0;
}

// ---------------------------------------------------------------------------
// Complex helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cd(double re, double im) { return make_double2(re, im); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cd(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return cd(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return cd(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    // scaled by the larger component of b (no overflow for any admittance)
    const double s = fmax(fabs(b.x), fabs(b.y));
    if (!(s > 0.0)) return cd(0.0, 0.0);
    const double bx = b.x / s, by = b.y / s, n = bx * bx + by * by;
    return cd((a.x * bx + a.y * by) / (s * n), (a.y * bx - a.x * by) / (s * n));
}

struct AcOut {
    double i_re, i_im, rms, res, i_err;
    int inner, outer;
};

// Work per frequency: 10 double2 vectors (x, r64, r, z, p, q, e, mlo, iw, chi)
// of na rows.
constexpr size_t kAcD2 = 10;

__device__ __forceinline__ double2 conj_free_dot(double2 a, double2 b) { return cmul(a, b); }

// z = M^-1 r over this thread's chains; accumulates r^T z (complex) and |r|^2.
__device__ __forceinline__ void ac_precond(uint32_t na, int chains, const double* __restrict__ glG,
                                           const double* __restrict__ grG, const double* __restrict__ grC,
                                           double w, const double2* __restrict__ mlo,
                                           const double2* __restrict__ iw, const double2* __restrict__ r,
                                           double2* __restrict__ z, uint32_t stride, double* acc) {
    for (uint32_t i = threadIdx.x; i < na; i += stride) {
        if (chains && glG[i] > 0.0) continue;
        uint32_t k = i;
        double2 y = r[k];
        z[k] = y;
        while (chains && grG[k] > 0.0 && k + 1 < na) {
            ++k;
            y = cadd(r[k], cmul(mlo[k], y));
            z[k] = y;
        }
        double2 zk = cmul(y, iw[k]);
        z[k] = zk;
        double2 t = conj_free_dot(r[k], zk);
        acc[0] += t.x;
        acc[1] += t.y;
        acc[2] += r[k].x * r[k].x + r[k].y * r[k].y;
        while (k > i) {
            --k;
            zk = cmul(cadd(z[k], cmul(cd(grG[k], w * grC[k]), zk)), iw[k]);
            z[k] = zk;
            t = conj_free_dot(r[k], zk);
            acc[0] += t.x;
            acc[1] += t.y;
            acc[2] += r[k].x * r[k].x + r[k].y * r[k].y;
        }
    }
}

// K x in difference form at row i: e_i x_i + sum_k Y_k (x_i - x_col) + chain links.
__device__ __forceinline__ double2 ac_row(uint32_t i, double w, const double2* __restrict__ x,
                                          const uint32_t* __restrict__ rowp, const uint32_t* __restrict__ col,
                                          const double* __restrict__ vG, const double* __restrict__ vC,
                                          const double* __restrict__ eG, const double* __restrict__ eC, int chains,
                                          const double* __restrict__ glG, const double* __restrict__ grG,
                                          const double* __restrict__ glC, const double* __restrict__ grC) {
    const double2 xi = x[i];
    double2 a = cmul(cd(eG[i], w * eC[i]), xi);
    for (uint32_t k = rowp[i], k1 = rowp[i + 1]; k < k1; ++k)
        a = cadd(a, cmul(cd(vG[k], w * vC[k]), csub(xi, x[col[k]])));
    if (chains) {
        if (glG[i] > 0.0) a = cadd(a, cmul(cd(glG[i], w * glC[i]), csub(xi, x[i - 1])));
        if (grG[i] > 0.0) a = cadd(a, cmul(cd(grG[i], w * grC[i]), csub(xi, x[i + 1])));
    }
    return a;
}

// One CTA per frequency: COCG in FP64 complex arithmetic, restarted from the
// true residual until it meets tol. The admittances of one network span up to
// ~1e12 (rod segments against contacts at the tunnelling range), beyond what
// FP32 vectors resolve.
//
// Unknown: x = chi - V, chi = 1 on the resistive clusters (G > 0 edges) tied to
// the source, 0 elsewhere; K x = K chi - b, the right-hand side formed in
// difference form (exact for 0 / 1 values). When the resistive network does
// not join the electrodes, the current at low frequency (~1e-14 of the
// electrode admittances) crosses capacitive links only and the source
// clusters sit at V = 1 - O(1e-14): V itself cannot carry 1 - V in FP64, x
// can. I = sum_i b_i (1 - chi_i + x_i).
template <int NT>
__global__ void __launch_bounds__(NT) k_ac_cocg(int nf, const double* __restrict__ wsc, uint32_t na,
                                                const uint32_t* __restrict__ rowp, const uint32_t* __restrict__ col,
                                                const double* __restrict__ vG, const double* __restrict__ vC,
                                                const double* __restrict__ eG, const double* __restrict__ eC,
                                                const double* __restrict__ cG, const double* __restrict__ cC,
                                                const double* __restrict__ ch64, int chains,
                                                const double* __restrict__ bG, const double* __restrict__ bC,
                                                const double* __restrict__ chi, double2* __restrict__ dwork,
                                                double tol, int max_inner, AcOut* __restrict__ out) {
    __shared__ double sh[4 * 40 + 8];
    const int f = blockIdx.x;
    if (f >= nf) return;
    const double w = wsc[f];
    double2* x = dwork + kAcD2 * na * (size_t)f;
    double2* rv = x + na;
    double2* r = rv + na;
    double2* z = r + na;
    double2* p = z + na;
    double2* q = p + na;
    double2* ee = q + na;
    double2* mlo = ee + na;
    double2* iw = mlo + na;
    double2* xc = iw + na;  // chi as complex values
    const double* glG = ch64;
    const double* grG = ch64 + na;
    const double* glC = ch64 + 2ull * na;
    const double* grC = ch64 + 3ull * na;
    AcOut o{};

    // Chain factors at this frequency.
    for (uint32_t i = threadIdx.x; i < na; i += NT) {
        if (chains && glG[i] > 0.0) continue;
        double2 gam = cd(cG[i], w * cC[i]);
        uint32_t k = i;
        mlo[k] = cd(0.0, 0.0);
        while (true) {
            const double2 g = chains ? cd(grG[k], w * grC[k]) : cd(0.0, 0.0);
            const double2 wk = cadd(g, gam);
            iw[k] = cdiv(cd(1.0, 0.0), wk);
            if (!(g.x > 0.0) || k + 1 >= na) break;
            mlo[k + 1] = cdiv(g, wk);
            gam = cadd(cd(cG[k + 1], w * cC[k + 1]), cdiv(cmul(g, gam), cadd(g, gam)));
            ++k;
        }
    }
    for (uint32_t i = threadIdx.x; i < na; i += NT) {
        x[i] = cd(0.0, 0.0);
        xc[i] = cd(chi[i], 0.0);
    }
    __syncthreads();  // chi staged
    double nrm[2] = {0.0, 0.0};  // |c|^2, |b|^2
    for (uint32_t i = threadIdx.x; i < na; i += NT) {
        const double2 b = cd(bG[i], w * bC[i]);
        const double2 c = csub(ac_row(i, w, xc, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC), b);
        rv[i] = c;
        nrm[0] += c.x * c.x + c.y * c.y;
        nrm[1] += b.x * b.x + b.y * b.y;
    }
    block_sum_k<NT, 2>(nrm, sh);
    // Convergence is judged against |b| (the scale of the Kirchhoff tool's
    // RMS column): |c| can fall below the rounding floor of the node
    // potentials (stiff rod segments times one ulp of V) at low frequency.
    const double bn = sqrt(nrm[1]);
    double rn = sqrt(nrm[0]);
    // Iterate to the rounding floor (restarts stop when the true residual no
    // longer halves); the point counts as converged when it is within tol.
    int inner_total = 0, outer = 0;
    for (; outer < 40; ++outer) {
        if (!(rn > 1e-15 * bn)) break;
        const double target = 1e-8;
        const double sc = 1.0 / rn;
        for (uint32_t i = threadIdx.x; i < na; i += NT) {
            r[i] = cd(rv[i].x * sc, rv[i].y * sc);
            ee[i] = cd(0.0, 0.0);
        }
        __syncthreads();  // r complete
        double acc[3] = {0.0, 0.0, 0.0};
        ac_precond(na, chains, glG, grG, grC, w, mlo, iw, r, z, NT, acc);
        block_sum_k<NT, 3>(acc, sh);
        double2 rho = cd(acc[0], acc[1]);
        const double r0 = sqrt(acc[2]);
        for (uint32_t i = threadIdx.x; i < na; i += NT) p[i] = z[i];
        int it = 0;
        double best = 1.0;  // recursive residual, relative to r0
        int best_it = 0;
        for (; it < max_inner; ++it) {
            __syncthreads();  // p complete
            double mu[2] = {0.0, 0.0};
            for (uint32_t i = threadIdx.x; i < na; i += NT) {
                const double2 a = ac_row(i, w, p, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC);
                q[i] = a;
                const double2 t = cmul(p[i], a);
                mu[0] += t.x;
                mu[1] += t.y;
            }
            block_sum_k<NT, 2>(mu, sh);
            if (!(fabs(mu[0]) + fabs(mu[1]) > 0.0)) break;
            const double2 alpha = cdiv(rho, cd(mu[0], mu[1]));
            for (uint32_t i = threadIdx.x; i < na; i += NT) {
                ee[i] = cadd(ee[i], cmul(alpha, p[i]));
                r[i] = csub(r[i], cmul(alpha, q[i]));
            }
            __syncthreads();  // r complete
            double a2[3] = {0.0, 0.0, 0.0};
            ac_precond(na, chains, glG, grG, grC, w, mlo, iw, r, z, NT, a2);
            block_sum_k<NT, 3>(a2, sh);
            const double rel = sqrt(a2[2]) / r0;
            if (rel <= target) { ++it; break; }
            if (rel < 0.5 * best) { best = rel; best_it = it; }
            if (it - best_it > 2000) { ++it; break; }  // the recursion has stalled
            const double2 rho_new = cd(a2[0], a2[1]);
            const double2 beta = cdiv(rho_new, rho);
            rho = rho_new;
            for (uint32_t i = threadIdx.x; i < na; i += NT) p[i] = cadd(z[i], cmul(beta, p[i]));
        }
        inner_total += it;
        __syncthreads();
        // candidate x + rn e (in z) and its true residual (in q), row order
        for (uint32_t i = threadIdx.x; i < na; i += NT) z[i] = cadd(x[i], cd(rn * ee[i].x, rn * ee[i].y));
        __syncthreads();
        double part = 0.0;
        for (uint32_t i = threadIdx.x; i < na; i += NT) {
            const double2 a = ac_row(i, w, z, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC);
            const double2 c = ac_row(i, w, xc, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC);
            const double2 ri = csub(csub(c, cd(bG[i], w * bC[i])), a);
            q[i] = ri;
            part += ri.x * ri.x + ri.y * ri.y;
        }
        const double rn_new = sqrt(block_sum<NT>(part, sh));
        // a step is kept only if it lowers the true residual: near the
        // rounding floor a restart can wander (the start V = chi may already
        // be below the floor of the recursion at low frequency)
        if (!(rn_new < rn)) { ++outer; break; }
        for (uint32_t i = threadIdx.x; i < na; i += NT) {
            x[i] = z[i];
            rv[i] = q[i];
        }
        __syncthreads();
        const bool stalled = !(rn_new < 0.5 * rn);
        rn = rn_new;
        if (it == 0 || stalled) { ++outer; break; }  // no further progress
    }
    // I = sum b (1 - chi + x); its first-order error is V^T r with V = chi - x
    // and r the last true residual of x (K symmetric: dI = b^T K^-1 r).
    double cur[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = threadIdx.x; i < na; i += NT) {
        const double2 t = cmul(cd(bG[i], w * bC[i]), cadd(cd(1.0 - chi[i], 0.0), x[i]));
        cur[0] += t.x;
        cur[1] += t.y;
        const double2 d = cmul(csub(cd(chi[i], 0.0), x[i]), rv[i]);
        cur[2] += d.x;
        cur[3] += d.y;
    }
    block_sum_k<NT, 4>(cur, sh);
    if (threadIdx.x == 0) {
        o.i_re = cur[0];
        o.i_im = cur[1];
        o.rms = rn;
        o.res = bn > 0 ? rn / bn : 0.0;
        o.i_err = sqrt(cur[2] * cur[2] + cur[3] * cur[3]);
        o.inner = inner_total;
        o.outer = outer;
        out[f] = o;
    }
}

// ---------------------------------------------------------------------------
// Direct form: banded complex-symmetric LDL^T per frequency.
//
// The active system is reordered by reverse Cuthill-McKee on the host (the
// networks of the tool are sparse and nearly one-dimensional: the jammed
// node network of 2 777 active nodes has bandwidth 30 after it), and every
// frequency's CTA assembles its band, factors it without pivoting (all
// admittances lie in the first quadrant, the matrix is complex symmetric and
// diagonally dominant in the sense that each diagonal is the sum of its row's
// off-diagonal admittances plus the electrode ones), and refines x on the
// difference-form residual as the oracle's refined LU does. This is the
// tool's own method (a direct factorisation per frequency) and does not
// stagnate on stiff networks. Band storage: row p of the reordered matrix
// holds A[p][p - o] for o = 0..b.
// ---------------------------------------------------------------------------
constexpr uint32_t kBandMax = 512;

template <int NT>
__global__ void __launch_bounds__(NT) k_ac_band(int nf, const double* __restrict__ wsc, uint32_t na, uint32_t b,
                                                const uint32_t* __restrict__ perm, const uint32_t* __restrict__ rowp,
                                                const uint32_t* __restrict__ col, const double* __restrict__ vG,
                                                const double* __restrict__ vC, const double* __restrict__ eG,
                                                const double* __restrict__ eC, const double* __restrict__ ch64,
                                                int chains, const double* __restrict__ bG,
                                                const double* __restrict__ bC, const double* __restrict__ chi,
                                                double2* __restrict__ bwork, double2* __restrict__ vwork,
                                                AcOut* __restrict__ out) {
    __shared__ double sh[4 * 40 + 8];
    __shared__ double2 lsh[kBandMax], ush[kBandMax];
    const int f = blockIdx.x;
    if (f >= nf) return;
    const double w = wsc[f];
    const size_t bw = (size_t)b + 1;
    double2* A = bwork + (size_t)f * na * bw;
    double2* x = vwork + (size_t)f * 5 * na;  // unknowns, original order
    double2* rv = x + na;                      // residual, original order
    double2* xc = rv + na;                     // chi
    double2* t = xc + na;                      // solve vector, reordered
    double2* xt = t + na;                      // candidate x
    const double* glG = ch64;
    const double* grG = ch64 + na;
    const double* glC = ch64 + 2ull * na;
    const double* grC = ch64 + 3ull * na;
    AcOut o{};
    // band assembly, one row per thread
    for (uint32_t i = threadIdx.x; i < na; i += NT) {
        const uint32_t p = perm[i];
        double2* row = A + (size_t)p * bw;
        for (uint32_t q = 1; q < bw; ++q) row[q] = cd(0.0, 0.0);
        double2 d = cd(eG[i], w * eC[i]);
        for (uint32_t k = rowp[i], k1 = rowp[i + 1]; k < k1; ++k) {
            const double2 y = cd(vG[k], w * vC[k]);
            d = cadd(d, y);
            const uint32_t q = perm[col[k]];
            if (q < p && p - q <= b) row[p - q] = csub(row[p - q], y);
        }
        if (chains) {
            if (glG[i] > 0.0) {
                const double2 y = cd(glG[i], w * glC[i]);
                d = cadd(d, y);
                const uint32_t q = perm[i - 1];
                if (q < p && p - q <= b) row[p - q] = csub(row[p - q], y);
            }
            if (grG[i] > 0.0) {
                const double2 y = cd(grG[i], w * grC[i]);
                d = cadd(d, y);
                const uint32_t q = perm[i + 1];
                if (q < p && p - q <= b) row[p - q] = csub(row[p - q], y);
            }
        }
        row[0] = d;
        x[i] = cd(0.0, 0.0);
        xc[i] = cd(chi[i], 0.0);
    }
    __syncthreads();
    // LDL^T, right-looking: column k scales by 1 / d_k, the trailing triangle
    // loses l_i (d_k l_j) = l_i A[j][j-k]
    for (uint32_t k = 0; k < na; ++k) {
        const double2 dk = A[(size_t)k * bw];
        const uint32_t m = min(b, na - 1 - k);
        for (uint32_t u = threadIdx.x; u < m; u += NT) {
            const double2 a = A[(size_t)(k + 1 + u) * bw + (u + 1)];
            ush[u] = a;
            lsh[u] = cdiv(a, dk);
        }
        __syncthreads();
        const uint32_t ntri = m * (m + 1) / 2;
        for (uint32_t v = threadIdx.x; v < ntri; v += NT) {
            uint32_t ii = (uint32_t)((sqrt(8.0 * v + 1.0) - 1.0) * 0.5);
            while ((ii + 1) * (ii + 2) / 2 <= v) ++ii;  // exact triangular root
            while (ii * (ii + 1) / 2 > v) --ii;
            const uint32_t jj = v - ii * (ii + 1) / 2;
            const uint32_t i = k + 1 + ii;
            double2* e = A + (size_t)i * bw + (ii - jj);
            *e = csub(*e, cmul(lsh[ii], ush[jj]));
        }
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < m; u += NT) A[(size_t)(k + 1 + u) * bw + (u + 1)] = lsh[u];
        __syncthreads();
    }
    // refinement on K x = K chi - b (x = chi - V), residual in difference form
    double rn = 0.0, bn = 0.0;
    {
        double nrm[2] = {0.0, 0.0};
        for (uint32_t i = threadIdx.x; i < na; i += NT) {
            const double2 bb = cd(bG[i], w * bC[i]);
            const double2 c = csub(ac_row(i, w, xc, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC), bb);
            rv[i] = c;
            nrm[0] += c.x * c.x + c.y * c.y;
            nrm[1] += bb.x * bb.x + bb.y * bb.y;
        }
        block_sum_k<NT, 2>(nrm, sh);
        rn = sqrt(nrm[0]);
        bn = sqrt(nrm[1]);
    }
    int steps = 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (; steps < 12 && rn > 1e-15 * bn; ++steps) {
        for (uint32_t i = threadIdx.x; i < na; i += NT) t[perm[i]] = rv[i];
        __syncthreads();
        if (warp == 0) {
            // forward: t_i -= l_ik t_k below the diagonal, column by column
            for (uint32_t k = 0; k < na; ++k) {
                const double2 tk = t[k];
                const uint32_t m = min(b, na - 1 - k);
                for (uint32_t u = lane; u < m; u += 32) {
                    const uint32_t i = k + 1 + u;
                    t[i] = csub(t[i], cmul(A[(size_t)i * bw + (u + 1)], tk));
                }
                __syncwarp();
            }
            for (uint32_t k = lane; k < na; k += 32) t[k] = cdiv(t[k], A[(size_t)k * bw]);
            __syncwarp();
            // backward: t_k -= sum_i l_ik t_i over the band below k
            for (uint32_t kk = na; kk-- > 0;) {
                const uint32_t m = min(b, na - 1 - kk);
                double2 acc = cd(0.0, 0.0);
                for (uint32_t u = lane; u < m; u += 32) {
                    const uint32_t i = kk + 1 + u;
                    acc = cadd(acc, cmul(A[(size_t)i * bw + (u + 1)], t[i]));
                }
#pragma unroll
                for (int s = 16; s > 0; s >>= 1) {
                    acc.x += __shfl_down_sync(0xffffffffu, acc.x, s);
                    acc.y += __shfl_down_sync(0xffffffffu, acc.y, s);
                }
                if (lane == 0) t[kk] = csub(t[kk], acc);
                __syncwarp();
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < na; i += NT) xt[i] = cadd(x[i], t[perm[i]]);
        __syncthreads();
        double part = 0.0;
        for (uint32_t i = threadIdx.x; i < na; i += NT) {
            const double2 a = ac_row(i, w, xt, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC);
            const double2 c = ac_row(i, w, xc, rowp, col, vG, vC, eG, eC, chains, glG, grG, glC, grC);
            const double2 ri = csub(csub(c, cd(bG[i], w * bC[i])), a);
            t[perm[i]] = ri;  // the solve vector is free again: hold the candidate residual
            part += ri.x * ri.x + ri.y * ri.y;
        }
        const double rn_new = sqrt(block_sum<NT>(part, sh));
        if (!(rn_new < rn)) { ++steps; break; }  // at the rounding floor
        for (uint32_t i = threadIdx.x; i < na; i += NT) {
            x[i] = xt[i];
            rv[i] = t[perm[i]];
        }
        __syncthreads();
        rn = rn_new;
    }
    double cur[4] = {0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = threadIdx.x; i < na; i += NT) {
        const double2 tt = cmul(cd(bG[i], w * bC[i]), cadd(cd(1.0 - chi[i], 0.0), x[i]));
        cur[0] += tt.x;
        cur[1] += tt.y;
        const double2 d = cmul(csub(cd(chi[i], 0.0), x[i]), rv[i]);
        cur[2] += d.x;
        cur[3] += d.y;
    }
    block_sum_k<NT, 4>(cur, sh);
    if (threadIdx.x == 0) {
        o.i_re = cur[0];
        o.i_im = cur[1];
        o.rms = rn;
        o.res = bn > 0 ? rn / bn : 0.0;
        o.i_err = sqrt(cur[2] * cur[2] + cur[3] * cur[3]);
        o.inner = steps;
        o.outer = steps;
        out[f] = o;
    }
}

// Reverse Cuthill-McKee order of the active system (CSR rows plus the chain
// links i -> i + 1): perm[old] = new; returns the bandwidth.
uint32_t rcm_order(uint32_t n, const std::vector<uint32_t>& rowp, const std::vector<uint32_t>& col,
                   const std::vector<char>& up, std::vector<uint32_t>* perm) {
    std::vector<uint32_t> deg(n, 0);
    for (uint32_t i = 0; i < n; ++i) deg[i] = rowp[i + 1] - rowp[i] + (up[i] ? 1 : 0) + (i > 0 && up[i - 1] ? 1 : 0);
    auto nbrs = [&](uint32_t i, std::vector<uint32_t>& out) {
        out.clear();
        for (uint32_t k = rowp[i]; k < rowp[i + 1]; ++k) out.push_back(col[k]);
        if (up[i]) out.push_back(i + 1);
        if (i > 0 && up[i - 1]) out.push_back(i - 1);
    };
    std::vector<int64_t> level(n, -1);
    std::vector<uint32_t> order;
    order.reserve(n);
    std::vector<char> done(n, 0);
    std::vector<uint32_t> nb, q;
    q.reserve(n);
    // Breadth-first sweep from s over nodes not yet ordered; returns the last
    // node reached. Only the ordering sweep (seq given) visits neighbours by
    // increasing degree; the two sweeps that look for a pseudo-peripheral
    // start need the level structure alone.
    auto bfs = [&](uint32_t s, std::vector<uint32_t>* seq) {
        q.assign(1, s);
        level[s] = 0;
        size_t h = 0;
        while (h < q.size()) {
            const uint32_t v = q[h++];
            nbrs(v, nb);
            if (seq)
                std::sort(nb.begin(), nb.end(),
                          [&](uint32_t a, uint32_t c) { return deg[a] != deg[c] ? deg[a] < deg[c] : a < c; });
            for (uint32_t u : nb)
                if (level[u] < 0 && !done[u]) { level[u] = level[v] + 1; q.push_back(u); }
        }
        if (seq) *seq = q;
        const uint32_t last = q.back();
        for (uint32_t v : q) level[v] = -1;  // q holds every node this sweep reached
        return last;
    };
    for (uint32_t s0 = 0; s0 < n; ++s0) {
        if (done[s0]) continue;
        uint32_t s = s0;  // pseudo-peripheral start: two sweeps from the component's first node
        s = bfs(s, nullptr);
        s = bfs(s, nullptr);
        std::vector<uint32_t> seq;
        bfs(s, &seq);
        for (uint32_t v : seq) { done[v] = 1; order.push_back(v); }
    }
    perm->assign(n, 0);
    for (uint32_t k = 0; k < n; ++k) (*perm)[order[n - 1 - k]] = k;
    uint32_t bwid = 0;
    for (uint32_t i = 0; i < n; ++i) {
        nbrs(i, nb);
        for (uint32_t j : nb) {
            const uint32_t a = (*perm)[i], c = (*perm)[j];
            bwid = std::max(bwid, a > c ? a - c : c - a);
        }
    }
    return bwid;
}

nf_status Engine::ac_spectrum(const nf_ac_net* net, const nf_ac_params& P, const double* freq, size_t nfreq,
                              nf_ac_point* out, nf_ac_stats* stats) {
    EventPair ev;
    NF_CK(ev.create());
    NF_CK(cudaEventRecord(ev.a, st));
    // Scales of the tool (kirchhoff.py:66-88), SI units.
    const double rc = P.r_cnt * 1e-6, dmin = P.delta_min * 1e-6;
    const double smin = kPi * rc * rc, smax = P.l_cnt * 1e-6 * 2.0 * rc;
    const double phi = P.phi_ev * kE;
    const double mphi = std::sqrt(2.0 * kMe * phi);
    const double Acoef = 1.0 / mphi * (kH / kE) * (kH / kE);
    const double Bcoef = 4.0 * kPi / kH * mphi;
    const double R0 = Acoef * std::exp(Bcoef * dmin) * dmin / smin;
    const double C0 = kEps0 * P.eps_r * smin / dmin;
    const double w0 = 1.0 / (R0 * C0);
    AcConst k{dmin, P.delta_tun * 1e-6, P.delta_eff * 1e-6, smin, smax, Bcoef, P.c_min, 2.0 * rc, P.own_radii};

    // Edges: [contacts | segments]; I / J node ids.
    uint32_t n = 0, mct = 0, ns = 0;
    const uint32_t *eI = nullptr, *eJ = nullptr;
    DBuf<uint32_t> uI, uJ;
    DBuf<double> uD, uS, uL, uA;
    std::vector<uint32_t> off(2, 0);
    std::vector<uint32_t> hI, hJ;
    uint32_t mchain = 0;  // first chain-link edge
    if (!net) {
        mct = (uint32_t)ct_off[1];
        if (int_valid) {
            n = (uint32_t)int_nodes;
            ns = (uint32_t)int_segs;
            eI = ieI.p;
            eJ = ieJ.p;
        } else {
            n = (uint32_t)rod_slots;
            eI = cI.p;
            eJ = cJ.p;
        }
        mchain = mct;
    } else {
        n = (uint32_t)net->n_nodes;
        mct = (uint32_t)net->n_contacts;
        ns = (uint32_t)net->n_segments;
        // General edges first (contacts, then segments that are not a first
        // link (i, i + 1)), chain links last.
        std::vector<char> seen(n + 1, 0);
        std::vector<uint32_t> chainI, chainJ, genI, genJ;
        std::vector<double> chainL, chainA, genL, genA;
        for (uint32_t s = 0; s < ns; ++s) {
            const uint32_t i = net->seg_i[s], j = net->seg_j[s];
            if (j == i + 1 && !seen[i]) {
                seen[i] = 1;
                chainI.push_back(i); chainJ.push_back(j); chainL.push_back(net->seg_l[s]); chainA.push_back(net->seg_a[s]);
            } else {
                genI.push_back(i); genJ.push_back(j); genL.push_back(net->seg_l[s]); genA.push_back(net->seg_a[s]);
            }
        }
        hI.assign(net->ct_i, net->ct_i + mct);
        hJ.assign(net->ct_j, net->ct_j + mct);
        hI.insert(hI.end(), genI.begin(), genI.end());
        hI.insert(hI.end(), chainI.begin(), chainI.end());
        hJ.insert(hJ.end(), genJ.begin(), genJ.end());
        hJ.insert(hJ.end(), chainJ.begin(), chainJ.end());
        mchain = mct + (uint32_t)genI.size();
        std::vector<double> hL(genL), hA(genA);
        hL.insert(hL.end(), chainL.begin(), chainL.end());
        hA.insert(hA.end(), chainA.begin(), chainA.end());
        const size_t m = hI.size();
        NF_CK(uI.ensure(m + 1));
        NF_CK(uJ.ensure(m + 1));
        NF_CK(uD.ensure(mct + 1));
        NF_CK(uS.ensure(mct + 1));
        NF_CK(uL.ensure(ns + 1));
        NF_CK(uA.ensure(ns + 1));
        NF_CK(cudaMemcpyAsync(uI.p, hI.data(), 4 * m, cudaMemcpyHostToDevice, st));
        NF_CK(cudaMemcpyAsync(uJ.p, hJ.data(), 4 * m, cudaMemcpyHostToDevice, st));
        if (mct) {
            NF_CK(cudaMemcpyAsync(uD.p, net->ct_d, 8ull * mct, cudaMemcpyHostToDevice, st));
            NF_CK(cudaMemcpyAsync(uS.p, net->ct_s, 8ull * mct, cudaMemcpyHostToDevice, st));
        }
        if (ns) {
            NF_CK(cudaMemcpyAsync(uL.p, hL.data(), 8ull * ns, cudaMemcpyHostToDevice, st));
            NF_CK(cudaMemcpyAsync(uA.p, hA.data(), 8ull * ns, cudaMemcpyHostToDevice, st));
        }
        eI = uI.p;
        eJ = uJ.p;
    }
    const uint32_t m = mct + ns;
    off[1] = n;
    NF_CK(acG.ensure(m + 1));
    NF_CK(acC.ensure(m + 1));
    if (!net) {
        if (mct)
            NF_LAUNCH(k_ac_contacts, grid_for(mct, 256), 256, 0, st)(mct, cI.p, cJ.p, cD.p, cS.p, dir.p, k, acG.p,
                                                                     acC.p);
        if (ns)
            NF_LAUNCH(k_ac_segs_g, grid_for(ns, 256), 256, 0, st)(ns, ieG.p + mct, R0, acG.p + mct, acC.p + mct);
    } else {
        if (mct) NF_LAUNCH(k_ac_contacts_net, grid_for(mct, 256), 256, 0, st)(mct, uD.p, uS.p, k, acG.p, acC.p);
        if (ns)
            NF_LAUNCH(k_ac_segs_la, grid_for(ns, 256), 256, 0, st)(ns, uL.p, uA.p, prm[0].rod_sigma, R0, acG.p + mct,
                                                                   acC.p + mct);
    }
    NF_CK(cudaGetLastError());
    Asm A;
    nf_status s = assemble(n, off, mchain, m, eI, eJ, acG.p, acC.p, &A);
    if (s != NF_OK) return s;
    uint64_t kept = 0;
    if (mct) {
        std::vector<double> hg(mct), hc(mct);
        NF_CK(cudaMemcpyAsync(hg.data(), acG.p, 8ull * mct, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(hc.data(), acC.p, 8ull * mct, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        for (uint32_t e = 0; e < mct; ++e) kept += (hg[e] > 0.0 || hc[e] > 0.0) ? 1 : 0;
    }
    const uint32_t na = A.na;
    // chi: 1 on the active rows whose resistive cluster (edges with G > 0) has
    // a resistive contact to the source.
    NF_CK(acchi.ensure(na + 1));
    {
        uint32_t* act = eflag.p;
        uint32_t* errw = eflag.p + n + 1;
        if (n) NF_LAUNCH(k_uf_init, grid_for(n, 256), 256, 0, st)(n, parent.p, cflag.p);
        if (m) {
            NF_LAUNCH(k_uf_union, grid_for(m, 256), 256, 0, st)(m, eI, eJ, acG.p, acG.p, parent.p, errw);
            NF_LAUNCH(k_uf_flags, grid_for(m, 256), 256, 0, st)(m, eI, eJ, acG.p, acG.p, parent.p, cflag.p, errw);
        }
        if (n) NF_LAUNCH(k_ac_chi, grid_for(n, 256), 256, 0, st)(n, act, aidx.p, parent.p, cflag.p, acchi.p, errw);
        NF_CK(cudaGetLastError());
        uint32_t herr = 0;
        NF_CK(cudaMemcpyAsync(&herr, errw, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        if (herr) { err = "union-find walk exceeded its bound"; return NF_ERR_TIMEOUT; }
    }
    const double tol = P.tol > 0 ? P.tol : 1e-10;
    const int max_inner = prm[0].solve_max_iter > 0 ? prm[0].solve_max_iter : 20000;
    // Direct form when the reordered band is narrow enough: bandwidth <= 512,
    // at most 1 GB of band and ~4e9 complex updates per frequency.
    uint32_t bandw = 0;
    bool direct = false;
    DBuf<uint32_t> dperm;
    if (na > 0) {
        std::vector<uint32_t> hrow(na + 1), hcol(A.nnz);
        std::vector<double> hgr(na);
        NF_CK(cudaMemcpyAsync(hrow.data(), rowp.p, sizeof(uint32_t) * (na + 1), cudaMemcpyDeviceToHost, st));
        if (A.nnz) NF_CK(cudaMemcpyAsync(hcol.data(), col.p, sizeof(uint32_t) * A.nnz, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(hgr.data(), chain64.p + na, sizeof(double) * na, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        std::vector<char> up(na, 0);
        if (A.chains)
            for (uint32_t a = 0; a + 1 < na; ++a) up[a] = hgr[a] > 0.0 ? 1 : 0;
        std::vector<uint32_t> hperm;
        bandw = rcm_order(na, hrow, hcol, up, &hperm);
        const bool fits = bandw <= kBandMax && (double)na * (bandw + 1) * sizeof(double2) <= 1e9 &&
                          (double)na * bandw * bandw <= 4e9;
        if (P.method == 1 && !fits) { err = "the reordered band is too wide for the direct form"; return NF_ERR_PARAM; }
        direct = P.method != 2 && fits;
        if (direct) {
            NF_CK(dperm.ensure(na));
            NF_CK(cudaMemcpyAsync(dperm.p, hperm.data(), sizeof(uint32_t) * na, cudaMemcpyHostToDevice, st));
        }
    }
    // Frequencies per launch: the work memory of the batch held to ~4 GB.
    const size_t per = direct ? ((size_t)na * (bandw + 1) + 5 * (size_t)na) * sizeof(double2)
                              : kAcD2 * sizeof(double2) * (size_t)std::max<uint32_t>(na, 1);
    const size_t batch = std::max<size_t>(1, std::min<size_t>(nfreq, (size_t)4e9 / std::max<size_t>(per, 1)));
    DBuf<double2> dw, bwk;
    DBuf<double> wd;
    DBuf<AcOut> od;
    bool conv = true;
    if (na > 0) {
        if (direct) {
            NF_CK(bwk.ensure((size_t)na * (bandw + 1) * batch));
            NF_CK(dw.ensure(5 * (size_t)na * batch));
        } else {
            NF_CK(dw.ensure(kAcD2 * (size_t)na * batch));
        }
        NF_CK(wd.ensure(batch));
        NF_CK(od.ensure(batch));
    }
    std::vector<double> hw(batch);
    std::vector<AcOut> ho(batch);
    for (size_t f0 = 0; f0 < nfreq; f0 += batch) {
        const size_t nb = std::min(batch, nfreq - f0);
        if (na > 0) {
            for (size_t j = 0; j < nb; ++j) hw[j] = 2.0 * kPi * freq[f0 + j] / w0;
            NF_CK(cudaMemcpyAsync(wd.p, hw.data(), 8 * nb, cudaMemcpyHostToDevice, st));
            if (direct)
                NF_LAUNCH(k_ac_band<256>, (unsigned)nb, 256, 0, st)(
                    (int)nb, wd.p, na, bandw, dperm.p, rowp.p, col.p, val64.p, valC64.p, diag64.p, diagC64.p,
                    chain64.p, A.chains ? 1 : 0, bvec.p, bvecC.p, acchi.p, bwk.p, dw.p, od.p);
            else
                NF_LAUNCH(k_ac_cocg<512>, (unsigned)nb, 512, 0, st)(
                    (int)nb, wd.p, na, rowp.p, col.p, val64.p, valC64.p, diag64.p, diagC64.p, cdiag.p, cdiagC.p,
                    chain64.p, A.chains ? 1 : 0, bvec.p, bvecC.p, acchi.p, dw.p, tol, max_inner, od.p);
            NF_CK(cudaGetLastError());
            NF_CK(cudaMemcpyAsync(ho.data(), od.p, sizeof(AcOut) * nb, cudaMemcpyDeviceToHost, st));
            NF_CK(cudaStreamSynchronize(st));
        }
        for (size_t j = 0; j < nb; ++j) {
            nf_ac_point& o = out[f0 + j];
            o = nf_ac_point{};
            o.freq = freq[f0 + j];
            if (na == 0) {  // no path between the electrodes: I = 0
                o.z_re = o.z_im = HUGE_VAL;
                o.converged = 1;
                continue;
            }
            const AcOut& h = ho[j];
            o.i_re = h.i_re;
            o.i_im = h.i_im;
            const double den = h.i_re * h.i_re + h.i_im * h.i_im;
            const double zs = R0 * P.l_box * 1e-6;
            o.z_re = den > 0 ? zs * h.i_re / den : HUGE_VAL;
            o.z_im = den > 0 ? zs * h.i_im / den : HUGE_VAL;  // -Im(1/I) = Im(I) / |I|^2
            o.rms = h.rms;
            o.residual = h.res;
            o.i_err = h.i_err;
            o.iters = h.inner;
            o.converged = h.res <= tol ? 1 : 0;
            if (!o.converged) conv = false;
        }
    }
    NF_CK(cudaEventRecord(ev.b, st));
    NF_CK(cudaEventSynchronize(ev.b));
    float ms = 0;
    NF_CK(cudaEventElapsedTime(&ms, ev.a, ev.b));
    if (stats) {
        stats->n_nodes = n;
        stats->n_active = na;
        stats->n_contacts = mct;
        stats->n_kept = kept;
        stats->n_segments = ns;
        stats->R0 = R0;
        stats->C0 = C0;
        stats->omega0 = w0;
        stats->ms = ms;
        stats->bandwidth = bandw;
        stats->direct = direct ? 1 : 0;
    }
    if (!conv) { err = "AC solve did not reach its tolerance at some frequency"; return NF_ERR_NOT_CONVERGED; }
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
