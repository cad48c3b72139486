// nf_solve.cu -- conductance network: assembly, mixed-precision solve, adjoint.
//
// Reference path replaced: the offline Kirchhoff tool (tools/kirchhoff/kirchhoff.py:
// 211-269 with MKL DSS, tools/kirchhoff/lib/solver.cpp:185-269). Rods are nodes
// (equipotential); a rod-rod contact is a conductance G = G0 exp(-(gap-d_c)/lambda),
// gap floored at d_c (kirchhoff.py:146-148); electrode contacts enter in Norton
// form: diag += G_src + G_snk, rhs = G_src (source at 1 V, sink at 0 V,
// kirchhoff.py:239-242). G_eff = sum_i G_src,i (1 - V_i) (kirchhoff.py:269).
//
// Only rods whose connected component touches both electrodes carry current, so
// only those are unknowns (the rest of the matrix is singular or irrelevant; the
// reference floors empty rows at 1, kirchhoff.py:240).
//
// Solve: preconditioned CG in FP32 on the FP32 copy of the matrix, inside
// iterative refinement whose residual b - K x is accumulated in FP64 from the
// FP64 matrix. One CTA per realisation, all reductions block-deterministic.
// K is applied as a Laplacian, (K x)_i = e_i x_i + sum_j G_ij (x_i - x_j) with
// e_i the electrode conductance, so that strong edges between nearly
// equipotential nodes do not cancel against the diagonal.
//
// Preconditioner: block Jacobi over chains. In the intra-rod network the nodes
// of a rod are consecutive and joined by rod segments that conduct 1e3-1e9 times
// better than a tunnelling contact; each such chain is solved exactly as a
// tridiagonal system (Thomas algorithm) whose diagonal also carries the
// node's contact and electrode conductances. A rod-level network has chains of
// one node, where this is plain Jacobi. The LDL^T pivots are formed as
// w_k = g_k + gamma_k, gamma_k = c_k + g_{k-1} gamma_{k-1} / (g_{k-1} + gamma_{k-1})
// (g: segment conductance to the next node, c: the node's other conductances),
// a sum of positive terms with no cancellation.
//
// Adjoint: the Laplacian is self-adjoint, so dG_eff/dG_e = (V_i - V_j)^2 with
// V_src = 1, V_snk = 0 (Thomson's principle); no second solve is needed.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "nf_engine.cuh"
#include "nf_graph.cuh"
#include "nf_bcr.cuh"

namespace nf {

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

__global__ void k_uf_init(uint32_t n, uint32_t* parent, uint32_t* flag) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    parent[i] = i;
    flag[i] = 0;
}

// The assembly's first launch: union-find roots, electrode accumulators
// vsrc / vsnk (2 n + 2 each), the active-count sentinel act[n] and the error
// word.
__global__ void k_asm_init(uint32_t n, uint32_t* __restrict__ parent, uint32_t* __restrict__ flag,
                           double* __restrict__ vsrc, double* __restrict__ vsnk, uint32_t* __restrict__ act,
                           uint32_t* __restrict__ errw) {
    const size_t nv = 2ull * n + 2;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
        vsrc[i] = 0.0;
        vsnk[i] = 0.0;
        if (i < n) {
            parent[i] = (uint32_t)i;
            flag[i] = 0;
        }
        if (i == 0) {
            act[n] = 0;
            *errw = 0;
        }
    }
}

// out[r] = aidx[off[r]] (active rows before realisation r), r <= R; out[R + 1]
// the error word.
__global__ void k_asm_bases(int R, const uint32_t* __restrict__ off, const uint32_t* __restrict__ aidx,
                            const uint32_t* __restrict__ errw, uint32_t* __restrict__ out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= R + 1; r += gridDim.x * blockDim.x)
        out[r] = r <= R ? aidx[off[r]] : *errw;
}

// An edge conducts unless the admittance form gives it G = C = 0 (an AC
// contact beyond the electrostatic range); without C every edge conducts.
__device__ __forceinline__ bool edge_on(const double* G, const double* C, uint32_t e) {
    return !C || G[e] > 0.0 || C[e] > 0.0;
}

__global__ void k_uf_union(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                           const double* __restrict__ G, const double* __restrict__ C, uint32_t* parent,
                           uint32_t* err) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    uint32_t j = J[e];
    if (j >= NF_SNK_ELEC || !edge_on(G, C, e)) return;
    uint32_t a = I[e], b = j;
    for (uint32_t it = 0; it < kFindCap; ++it) {
        a = uf_find(parent, a, err);
        b = uf_find(parent, b, err);
        if (a == b) return;
        if (a < b) { uint32_t t = a; a = b; b = t; }
        if (atomicCAS(&parent[a], a, b) == a) return;  // hook larger root under smaller
    }
    atomicExch(err, 1u);
}

__global__ void k_uf_flags(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                           const double* __restrict__ G, const double* __restrict__ C, uint32_t* parent,
                           uint32_t* flag, uint32_t* err) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    uint32_t j = J[e];
    if (j < NF_SNK_ELEC || !edge_on(G, C, e)) return;
    uint32_t r = uf_find(parent, I[e], err);
    atomicOr(&flag[r], j == NF_SRC_ELEC ? 1u : 2u);
}

// Active (current-carrying) rods; per-rod source / sink conductance.
__global__ void k_active(uint32_t n, uint32_t* parent, const uint32_t* __restrict__ flag, uint32_t* __restrict__ act,
                         uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    act[i] = flag[uf_find(parent, i, err)] == 3u ? 1u : 0u;
}

// Electrode admittance per node (s: source, t: sink; sC, tC the capacitive
// parts when C is given), summed over the node's electrode edges in edge
// order: a node may carry several (buffer-layer electrodes give one contact
// per image rod), so the edges are listed per node, sorted and added in order.
__global__ void k_edeg(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                       const double* __restrict__ G, const double* __restrict__ C, uint32_t* __restrict__ ecnt) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m || J[e] < NF_SNK_ELEC || !edge_on(G, C, e)) return;
    atomicAdd(&ecnt[I[e]], 1u);
}

__global__ void k_efill(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                        const double* __restrict__ G, const double* __restrict__ C, const uint32_t* __restrict__ eoff,
                        uint32_t* __restrict__ ecur, uint32_t* __restrict__ elist) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m || J[e] < NF_SNK_ELEC || !edge_on(G, C, e)) return;
    const uint32_t i = I[e];
    elist[eoff[i] + atomicAdd(&ecur[i], 1u)] = e;
}

__global__ void k_esum(uint32_t n, const uint32_t* __restrict__ eoff, uint32_t* __restrict__ elist,
                       const uint32_t* __restrict__ J, const double* __restrict__ G, const double* __restrict__ C,
                       double* __restrict__ s, double* __restrict__ t, double* __restrict__ sC,
                       double* __restrict__ tC) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p0 = eoff[i], p1 = eoff[i + 1];
    if (p0 == p1) return;
    for (uint32_t k = p0 + 1; k < p1; ++k) {
        const uint32_t v = elist[k];
        uint32_t q = k;
        while (q > p0 && elist[q - 1] > v) { elist[q] = elist[q - 1]; --q; }
        elist[q] = v;
    }
    double gs = 0.0, gt = 0.0, cs = 0.0, ct = 0.0;
    for (uint32_t k = p0; k < p1; ++k) {
        const uint32_t e = elist[k];
        if (J[e] == NF_SRC_ELEC) { gs += G[e]; if (C) cs += C[e]; }
        else { gt += G[e]; if (C) ct += C[e]; }
    }
    s[i] = gs;
    t[i] = gt;
    if (C) { sC[i] = cs; tC[i] = ct; }
}

__global__ void k_deg(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                      const double* __restrict__ G, const double* __restrict__ C, const uint32_t* __restrict__ act,
                      const uint32_t* __restrict__ aidx, uint32_t* __restrict__ deg) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    uint32_t j = J[e];
    if (j >= NF_SNK_ELEC || !edge_on(G, C, e)) return;
    uint32_t i = I[e];
    if (!act[i]) return;  // both ends share a component
    atomicAdd(&deg[aidx[i]], 1u);
    atomicAdd(&deg[aidx[j]], 1u);
}

__global__ void k_fill(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                       const double* __restrict__ G, const double* __restrict__ C, const uint32_t* __restrict__ act,
                       const uint32_t* __restrict__ aidx, const uint32_t* __restrict__ rowp, uint32_t* __restrict__ cur,
                       uint32_t* __restrict__ col, double* __restrict__ v64, double* __restrict__ vC64) {
    uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    uint32_t j = J[e];
    if (j >= NF_SNK_ELEC || !edge_on(G, C, e)) return;
    uint32_t i = I[e];
    if (!act[i]) return;
    uint32_t a = aidx[i], b = aidx[j];
    uint32_t qa = rowp[a] + atomicAdd(&cur[a], 1u);
    uint32_t qb = rowp[b] + atomicAdd(&cur[b], 1u);
    col[qa] = b; v64[qa] = G[e];
    col[qb] = a; v64[qb] = G[e];
    if (C) { vC64[qa] = C[e]; vC64[qb] = C[e]; }
}

// Chain links (edges [mc, m)): node j = i + 1 of the same rod, both active or
// neither. gr[a] links row a to row a + 1, gl[a + 1] the same link seen from
// below.
// With C, the capacitive parts go to glC / grC (ch64 + 2 na, + 3 na).
__global__ void k_chain_links(uint32_t mc, uint32_t m, const uint32_t* __restrict__ I,
                              const uint32_t* __restrict__ J, const double* __restrict__ G,
                              const double* __restrict__ C, const uint32_t* __restrict__ act,
                              const uint32_t* __restrict__ aidx, uint32_t na, double* __restrict__ ch64,
                              uint32_t* err) {
    uint32_t e = mc + blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const uint32_t i = I[e], j = J[e];
    if (!act[i] || !edge_on(G, C, e)) return;
    const uint32_t a = aidx[i];
    if (j != i + 1 || !act[j] || aidx[j] != a + 1) { atomicExch(err, 2u); return; }
    ch64[a + na] = G[e];
    ch64[a + 1] = G[e];
    if (C) {
        ch64[3ull * na + a] = C[e];
        ch64[2ull * na + a + 1] = C[e];
    }
}

// Sort each row by (column, G, C) (deterministic SpMV order whatever order the
// atomics filled it in), FP32 copies, electrode conductance e = s + t, the
// row's non-chain conductance c = e + sum_k G_k, rhs b = s; with C the same
// for the capacitive parts (eC, cC, bC).
__global__ void k_rows(uint32_t nslot, const uint32_t* __restrict__ act, const uint32_t* __restrict__ aidx,
                       const uint32_t* __restrict__ rowp, uint32_t* __restrict__ col, double* __restrict__ v64,
                       double* __restrict__ vC64, float* __restrict__ v32, const double* __restrict__ s,
                       const double* __restrict__ t, const double* __restrict__ sC, const double* __restrict__ tC,
                       double* __restrict__ e64, float* __restrict__ e32, double* __restrict__ c64,
                       double* __restrict__ b, double* __restrict__ eC64, double* __restrict__ cC64,
                       double* __restrict__ bC) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot || !act[i]) return;
    uint32_t a = aidx[i];
    uint32_t p0 = rowp[a], p1 = rowp[a + 1];
    const bool ac = vC64 != nullptr;
    for (uint32_t k = p0 + 1; k < p1; ++k) {
        const uint32_t c = col[k];
        const double v = v64[k], w = ac ? vC64[k] : 0.0;
        uint32_t q = k;
        while (q > p0) {
            const uint32_t cp = col[q - 1];
            const double vp = v64[q - 1], wp = ac ? vC64[q - 1] : 0.0;
            if (!(cp > c || (cp == c && (vp > v || (vp == v && wp > w))))) break;
            col[q] = cp; v64[q] = vp;
            if (ac) vC64[q] = wp;
            --q;
        }
        col[q] = c;
        v64[q] = v;
        if (ac) vC64[q] = w;
    }
    const double el = s[i] + t[i];
    double c = el;
    for (uint32_t k = p0; k < p1; ++k) { c += v64[k]; v32[k] = (float)v64[k]; }
    e64[a] = el;
    e32[a] = (float)el;
    c64[a] = c;
    b[a] = s[i];
    if (ac) {
        const double elC = sC[i] + tC[i];
        double cc = elC;
        for (uint32_t k = p0; k < p1; ++k) cc += vC64[k];
        eC64[a] = elC;
        cC64[a] = cc;
        bC[a] = sC[i];
    }
}

// Tridiagonal factors per chain, from its first row (gl == 0): FP32 copies of
// the links, the forward multipliers mlo_k = g_{k-1} / w_{k-1} and 1 / w_k.
// ch32 layout: [gl | gr | mlo | iw], na entries each.
__global__ void k_chain_factor(uint32_t na, const double* __restrict__ gl, const double* __restrict__ gr,
                               const double* __restrict__ c64, float* __restrict__ ch32) {
    const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= na || gl[a] > 0.0) return;
    float* gl32 = ch32;
    float* gr32 = ch32 + na;
    float* mlo = ch32 + 2ull * na;
    float* iw = ch32 + 3ull * na;
    double gam = c64[a];
    uint32_t k = a;
    gl32[a] = 0.f;
    mlo[a] = 0.f;
    while (true) {
        const double g = gr[k];
        const double w = g + gam;
        iw[k] = w > 0.0 ? (float)(1.0 / w) : 0.f;
        gr32[k] = (float)g;
        if (!(g > 0.0) || k + 1 >= na) break;
        const uint32_t k1 = k + 1;
        gl32[k1] = (float)g;
        mlo[k1] = (float)(g / w);
        gam = c64[k1] + g * gam / (g + gam);
        k = k1;
    }
}

struct CgOut {
    double G, res;
    int outer, inner, n;
    int pad;
};

// z = M^-1 r on this thread's chains (rows i with gl[i] == 0 start one): a
// forward sweep y_k = r_k + mlo_k y_{k-1}, then z_k = (y_k + g_k z_{k+1}) / w_k.
// Accumulates r.z and r.r over the chain's rows.
__device__ __forceinline__ void chain_precond(uint32_t n, const float* __restrict__ gl, const float* __restrict__ gr,
                                              const float* __restrict__ mlo, const float* __restrict__ iw,
                                              const float* __restrict__ r, float* __restrict__ z, uint32_t stride,
                                              float* rz, float* rr) {
    for (uint32_t i = threadIdx.x; i < n; i += stride) {
        if (gl[i] != 0.f) continue;
        uint32_t k = i;
        float y = r[k];
        z[k] = y;
        while (gr[k] > 0.f && k + 1 < n) {
            ++k;
            y = r[k] + mlo[k] * y;
            z[k] = y;
        }
        float zk = y * iw[k];
        z[k] = zk;
        *rz += r[k] * zk;
        *rr += r[k] * r[k];
        while (k > i) {
            --k;
            zk = (z[k] + gr[k] * zk) * iw[k];
            z[k] = zk;
            *rz += r[k] * zk;
            *rr += r[k] * r[k];
        }
    }
}

// One CTA per realisation. work: 5 float vectors (r, z, p, q, e) per active row.
// e64 / e32: electrode conductance per row; CSR values are the conductances
// G > 0; ch64 = [gl | gr] and ch32 = [gl | gr | mlo | iw] hold the chain links
// and factors (na rows each) when chains != 0.
template <int NT>
__global__ void __launch_bounds__(NT) k_cg(int R, const uint32_t* __restrict__ abase,
                                           const uint32_t* __restrict__ rowp, const uint32_t* __restrict__ col,
                                           const float* __restrict__ v32, const double* __restrict__ v64,
                                           const float* __restrict__ e32, const double* __restrict__ e64,
                                           const double* __restrict__ ch64, const float* __restrict__ ch32,
                                           uint32_t na, int chains, const double* __restrict__ b,
                                           double* __restrict__ x, double* __restrict__ r64, float* __restrict__ work,
                                           double tol, int max_inner, CgOut* __restrict__ out) {
    __shared__ double sh[96];
    const int rr = blockIdx.x;
    if (rr >= R) return;
    const uint32_t base = abase[rr], n = abase[rr + 1] - base;
    float* w_r = work + 5ull * base;
    float* w_z = w_r + n;
    float* w_p = w_z + n;
    float* w_q = w_p + n;
    float* w_e = w_q + n;
    CgOut o{};
    o.n = (int)n;
    if (n == 0) {
        if (threadIdx.x == 0) out[rr] = o;
        return;
    }
    const double* bb = b + base;
    double* xx = x + base;
    double* rv = r64 + base;
    const float* gl32 = ch32 + base;
    const float* gr32 = ch32 + na + base;
    const float* mlo = ch32 + 2ull * na + base;
    const float* iw = ch32 + 3ull * na + base;
    const double* gl64 = ch64 + base;
    const double* gr64 = ch64 + na + base;
    double part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        xx[i] = 0.0;
        rv[i] = bb[i];
        part += bb[i] * bb[i];
    }
    const double bn = sqrt(block_sum<NT>(part, sh));
    double rn = bn;
    int inner_total = 0, outer = 0;
    const float inner_tol = 1e-4f;
    for (; outer < 40; ++outer) {
        if (!(rn > tol * bn)) break;
        const float sc = (float)(1.0 / rn);
        float prz = 0.f, prr = 0.f;
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            const float ri = (float)rv[i] * sc;
            w_r[i] = ri;
            w_e[i] = 0.f;
            if (!chains) {
                const float zi = ri * iw[i];
                w_z[i] = zi;
                prz += ri * zi;
                prr += ri * ri;
            }
        }
        if (chains) {
            __syncthreads();  // r complete
            chain_precond(n, gl32, gr32, mlo, iw, w_r, w_z, NT, &prz, &prr);
        }
        double rz, rr2;
        block_sum2<NT>(prz, prr, sh, &rz, &rr2);
        for (uint32_t i = threadIdx.x; i < n; i += NT) w_p[i] = w_z[i];
        const double r0 = sqrt(rr2);
        int it = 0;
        for (; it < max_inner; ++it) {
            __syncthreads();  // p complete
            float ppq = 0.f;
            for (uint32_t i = threadIdx.x; i < n; i += NT) {
                const uint32_t g = base + i;
                const float pi = w_p[i];
                float acc = e32[g] * pi;
                for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) acc += v32[k] * (pi - w_p[col[k] - base]);
                if (chains) {
                    const float a = gl32[i], c = gr32[i];
                    if (a != 0.f) acc += a * (pi - w_p[i - 1]);
                    if (c != 0.f) acc += c * (pi - w_p[i + 1]);
                }
                w_q[i] = acc;
                ppq += pi * acc;
            }
            const double pq = block_sum<NT>((double)ppq, sh);
            if (!(pq > 0.0)) break;
            const float alpha = (float)(rz / pq);
            float qz = 0.f, qr = 0.f;
            for (uint32_t i = threadIdx.x; i < n; i += NT) {
                w_e[i] += alpha * w_p[i];
                const float ri = w_r[i] - alpha * w_q[i];
                w_r[i] = ri;
                if (!chains) {
                    const float zi = ri * iw[i];
                    w_z[i] = zi;
                    qz += ri * zi;
                    qr += ri * ri;
                }
            }
            if (chains) {
                __syncthreads();  // r complete
                chain_precond(n, gl32, gr32, mlo, iw, w_r, w_z, NT, &qz, &qr);
            }
            double rz_new, rr_new;
            block_sum2<NT>(qz, qr, sh, &rz_new, &rr_new);
            if (sqrt(rr_new) <= inner_tol * r0) { ++it; break; }
            const float beta = (float)(rz_new / rz);
            rz = rz_new;
            for (uint32_t i = threadIdx.x; i < n; i += NT) w_p[i] = w_z[i] + beta * w_p[i];
        }
        inner_total += it;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += NT) xx[i] += rn * (double)w_e[i];
        __syncthreads();
        // FP64 residual in row order.
        part = 0.0;
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            const uint32_t g = base + i;
            const double xi = xx[i];
            double acc = e64[g] * xi;
            for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) acc += v64[k] * (xi - xx[col[k] - base]);
            if (chains) {
                const double a = gl64[i], c = gr64[i];
                if (a != 0.0) acc += a * (xi - xx[i - 1]);
                if (c != 0.0) acc += c * (xi - xx[i + 1]);
            }
            const double ri = bb[i] - acc;
            rv[i] = ri;
            part += ri * ri;
        }
        rn = sqrt(block_sum<NT>(part, sh));
        if (it == 0) break;  // no progress possible
    }
    part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) part += bb[i] * (1.0 - xx[i]);
    const double G = block_sum<NT>(part, sh);
    if (threadIdx.x == 0) {
        o.G = G;
        o.res = bn > 0 ? rn / bn : 0.0;
        o.outer = outer;
        o.inner = inner_total;
        out[rr] = o;
    }
}

// Voltages per rod; outside the source-sink network, components touching only
// the source sit at 1 V and all others at 0 V (no current flows there).
__global__ void k_scatter_v(uint32_t nslot, const uint32_t* __restrict__ act, const uint32_t* __restrict__ aidx,
                            const double* __restrict__ x, uint32_t* parent, const uint32_t* __restrict__ flag,
                            double* __restrict__ volt, uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot) return;
    volt[i] = act[i] ? x[aidx[i]] : (flag[uf_find(parent, i, err)] == 1u ? 1.0 : 0.0);
}

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

nf_status Engine::solve() {
    if (!contacts_valid) { err = "no contacts: run nf_contacts first"; return NF_ERR_STATE; }
    if (int_valid)
        return solve_graph((uint32_t)int_nodes, int_off, int_count, (uint32_t)(int_edges - int_segs),
                           (uint32_t)int_edges, ieI.p, ieJ.p, ieG.p);
    std::vector<uint32_t> off(R + 1), nodes(R);
    for (int r = 0; r < R; ++r) { off[r] = hreal[r].rod_off; nodes[r] = count[r]; }
    off[R] = (uint32_t)rod_slots;
    return solve_graph((uint32_t)rod_slots, off, nodes, (uint32_t)ct_off[R], (uint32_t)ct_off[R], cI.p, cJ.p, cG.p);
}

// Active-set system of a graph of n nodes (realisation r owns nodes
// [off[r], off[r+1])) and m edges (I, J, G[, C]); J may be NF_SRC_ELEC /
// NF_SNK_ELEC; edges [mc, m) are chain links (J = I + 1, same rod). Only nodes
// whose component touches both electrodes are unknowns. With C (admittance
// form) an edge with G = C = 0 is absent, and the capacitive parts are
// assembled beside the conductances (valC64, diagC64, cdiagC, bvecC, chain64
// [gl | gr | glC | grC]).
nf_status Engine::assemble(uint32_t n, const std::vector<uint32_t>& off, uint32_t mc, uint32_t m,
                           const uint32_t* eI, const uint32_t* eJ, const double* eG, const double* eC, Asm* out) {
    const int RR = (int)off.size() - 1;
    const uint32_t nslot = n;
    const bool ac = eC != nullptr;
    NF_CK(parent.ensure(nslot + 1));
    NF_CK(cflag.ensure(nslot + 1));
    NF_CK(aidx.ensure(nslot + 1));
    NF_CK(eflag.ensure(nslot + 2));  // act[] + error word
    NF_CK(vsrc.ensure(2ull * nslot + 2));  // [s | sC]
    NF_CK(vsnk.ensure(2ull * nslot + 2));  // [t | tC]
    uint32_t* act = eflag.p;
    uint32_t* errw = eflag.p + nslot + 1;
    double* sC = vsrc.p + nslot + 1;
    double* tC = vsnk.p + nslot + 1;
    NF_LAUNCH(k_asm_init, std::min(grid_for(2ull * nslot + 2, 256), 4096u), 256, 0, st)(nslot, parent.p, cflag.p,
                                                                                       vsrc.p, vsnk.p, act, errw);
    if (m) {
        NF_LAUNCH(k_uf_union, grid_for(m, 256), 256, 0, st)(m, eI, eJ, eG, eC, parent.p, errw);
        NF_LAUNCH(k_uf_flags, grid_for(m, 256), 256, 0, st)(m, eI, eJ, eG, eC, parent.p, cflag.p, errw);
    }
    if (nslot) NF_LAUNCH(k_active, grid_for(nslot, 256), 256, 0, st)(nslot, parent.p, cflag.p, act, errw);
    NF_CK(cudaGetLastError());
    nf_status s = scan_u32(act, aidx.p, nslot + 1);
    if (s != NF_OK) return s;
    // Active count per realisation (aidx at the node-range boundaries) and
    // the error word: one gather, one copy through the pinned buffer.
    {
        nf_status sp = ensure_pinned(sizeof(uint32_t) * (2 * (size_t)RR + 4));
        if (sp != NF_OK) return sp;
    }
    NF_CK(asmoff.ensure(2 * (size_t)RR + 4));
    uint32_t* hp = reinterpret_cast<uint32_t*>(hpin);
    std::memcpy(hp, off.data(), sizeof(uint32_t) * (RR + 1));
    NF_CK(cudaMemcpyAsync(asmoff.p, hp, sizeof(uint32_t) * (RR + 1), cudaMemcpyHostToDevice, st));
    NF_LAUNCH(k_asm_bases, grid_for((size_t)RR + 2, 256), 256, 0, st)(RR, asmoff.p, aidx.p, errw,
                                                                      asmoff.p + RR + 1);
    NF_CK(cudaMemcpyAsync(hp + RR + 1, asmoff.p + RR + 1, sizeof(uint32_t) * (RR + 2), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    out->habase.assign(hp + RR + 1, hp + 2 * RR + 2);
    uint32_t herr = hp[2 * RR + 2];
    if (herr) { err = "union-find walk exceeded its bound"; return NF_ERR_TIMEOUT; }
    const uint32_t na = out->habase[RR];
    out->na = na;
    out->chains = m > mc;
    if (na == 0) {  // no component joins both electrodes: nothing to assemble
        out->nnz = 0;
        return NF_OK;
    }
    // electrode admittance per node
    NF_CK(ecnt.ensure(nslot + 1));
    NF_CK(eoff.ensure(nslot + 1));
    NF_CK(elist.ensure((size_t)m + 1));
    NF_CK(cudaMemsetAsync(ecnt.p, 0, sizeof(uint32_t) * (nslot + 1), st));
    if (m) NF_LAUNCH(k_edeg, grid_for(m, 256), 256, 0, st)(m, eI, eJ, eG, eC, ecnt.p);
    NF_CK(cudaGetLastError());
    {
        nf_status se = scan_u32(ecnt.p, eoff.p, nslot + 1);
        if (se != NF_OK) return se;
    }
    NF_CK(cudaMemsetAsync(ecnt.p, 0, sizeof(uint32_t) * (nslot + 1), st));  // reuse as cursor
    if (m) NF_LAUNCH(k_efill, grid_for(m, 256), 256, 0, st)(m, eI, eJ, eG, eC, eoff.p, ecnt.p, elist.p);
    if (nslot)
        NF_LAUNCH(k_esum, grid_for(nslot, 256), 256, 0, st)(nslot, eoff.p, elist.p, eJ, eG, eC, vsrc.p, vsnk.p, sC, tC);
    NF_CK(cudaGetLastError());
    NF_CK(deg.ensure(na + 1));
    NF_CK(rowp.ensure(na + 1));
    NF_CK(cudaMemsetAsync(deg.p, 0, sizeof(uint32_t) * (na + 1), st));
    if (mc) NF_LAUNCH(k_deg, grid_for(mc, 256), 256, 0, st)(mc, eI, eJ, eG, eC, act, aidx.p, deg.p);
    NF_CK(cudaGetLastError());
    out->chains = m > mc;
    const size_t nch = (ac ? 4ull : 2ull) * na + 4;
    NF_CK(chain64.ensure(nch));
    NF_CK(chain32.ensure(4ull * na + 4));
    NF_CK(cudaMemsetAsync(chain64.p, 0, sizeof(double) * nch, st));
    if (out->chains)
        NF_LAUNCH(k_chain_links, grid_for(m - mc, 256), 256, 0, st)(mc, m, eI, eJ, eG, eC, act, aidx.p, na, chain64.p,
                                                                   errw);
    NF_CK(cudaGetLastError());
    s = scan_u32(deg.p, rowp.p, na + 1);
    if (s != NF_OK) return s;
    NF_CK(cudaMemcpyAsync(hp, rowp.p + na, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaMemcpyAsync(hp + 1, errw, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    const uint32_t nnz = hp[0];
    herr = hp[1];
    if (herr) { err = "chain link between non-consecutive active nodes"; return NF_ERR_STATE; }
    out->nnz = nnz;
    NF_CK(col.ensure(nnz + 1));
    NF_CK(val64.ensure(nnz + 1));
    NF_CK(val32.ensure(nnz + 1));
    NF_CK(diag64.ensure(na + 1));
    NF_CK(diag32.ensure(na + 1));
    NF_CK(cdiag.ensure(na + 1));
    NF_CK(bvec.ensure(na + 1));
    if (ac) {
        NF_CK(valC64.ensure(nnz + 1));
        NF_CK(diagC64.ensure(na + 1));
        NF_CK(cdiagC.ensure(na + 1));
        NF_CK(bvecC.ensure(na + 1));
    }
    NF_CK(cudaMemsetAsync(deg.p, 0, sizeof(uint32_t) * (na + 1), st));  // reuse as cursor
    if (mc)
        NF_LAUNCH(k_fill, grid_for(mc, 256), 256, 0, st)(mc, eI, eJ, eG, eC, act, aidx.p, rowp.p, deg.p, col.p,
                                                         val64.p, ac ? valC64.p : nullptr);
    if (nslot)
        NF_LAUNCH(k_rows, grid_for(nslot, 256), 256, 0, st)(nslot, act, aidx.p, rowp.p, col.p, val64.p,
                                                 ac ? valC64.p : nullptr, val32.p, vsrc.p, vsnk.p, sC, tC, diag64.p,
                                                 diag32.p, cdiag.p, bvec.p, ac ? diagC64.p : nullptr,
                                                 ac ? cdiagC.p : nullptr, ac ? bvecC.p : nullptr);
    NF_CK(cudaGetLastError());
    return NF_OK;
}

// Laplacian solve on the graph (see assemble); node voltages land in volt.
// ---------------------------------------------------------------------------
// Direct form: banded LDL^T per realisation.
//
// The rod networks are sparse and nearly one-dimensional between the
// electrodes: after reverse Cuthill-McKee (on the host, per realisation) the
// jammed box's 1 231 active rods have bandwidth 28, against ~800 PCG
// iterations of a stiff system (tunnelling conductances spread over orders
// of magnitude). One CTA per realisation assembles its band (row p holds
// A[p][p - o], o = 0..b), factors it without pivoting (the matrix is
// symmetric positive definite: each diagonal is its row's conductances plus
// the electrode ones), and refines x on the FP64 difference-form residual
// until it stops falling. Forward and backward substitution run on one warp.
// ---------------------------------------------------------------------------
constexpr uint32_t kDcBandMax = 512;

template <int NT>
__global__ void __launch_bounds__(NT) k_dc_band(int R, const uint32_t* __restrict__ abase,
                                                const unsigned long long* __restrict__ boff,
                                                const uint32_t* __restrict__ bwid, const uint32_t* __restrict__ permL,
                                                const uint32_t* __restrict__ rowp, const uint32_t* __restrict__ col,
                                                const double* __restrict__ v64, const double* __restrict__ e64,
                                                const double* __restrict__ ch64, int chains,
                                                const double* __restrict__ b, double* __restrict__ x,
                                                double* __restrict__ r64, double* __restrict__ band,
                                                double* __restrict__ work, double tol, CgOut* __restrict__ out) {
    __shared__ double sh[96];
    __shared__ double lsh[kDcBandMax], ush[kDcBandMax];
    const int rr = blockIdx.x;
    if (rr >= R) return;
    const uint32_t base = abase[rr], n = abase[rr + 1] - base, bw = bwid[rr], bs = bw + 1;
    CgOut o{};
    o.n = (int)n;
    if (n == 0) {
        if (threadIdx.x == 0) out[rr] = o;
        return;
    }
    double* A = band + boff[rr];
    const uint32_t* perm = permL + base;
    const double* bb = b + base;
    double* xx = x + base;
    double* rv = r64 + base;
    double* t = work + base;                 // solve vector, reordered
    double* xt = work + abase[R] + base;     // candidate x
    const double* gl64 = ch64 + base;
    const double* gr64 = ch64 + abase[R] + base;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        const uint32_t g = base + i, p = perm[i];
        double* row = A + (size_t)p * bs;
        for (uint32_t q = 1; q < bs; ++q) row[q] = 0.0;
        double d = e64[g];
        for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) {
            d += v64[k];
            const uint32_t q = perm[col[k] - base];
            if (q < p && p - q <= bw) row[p - q] -= v64[k];
        }
        if (chains) {
            if (gl64[i] > 0.0) {
                d += gl64[i];
                const uint32_t q = perm[i - 1];
                if (q < p && p - q <= bw) row[p - q] -= gl64[i];
            }
            if (gr64[i] > 0.0) {
                d += gr64[i];
                const uint32_t q = perm[i + 1];
                if (q < p && p - q <= bw) row[p - q] -= gr64[i];
            }
        }
        row[0] = d;
        xx[i] = 0.0;
    }
    __syncthreads();
    // LDL^T, right-looking: column k scaled by 1 / d_k, the trailing triangle
    // loses l_i (d_k l_j) = l_i A[j][j - k]
    for (uint32_t k = 0; k < n; ++k) {
        const double dk = A[(size_t)k * bs];
        const uint32_t m = min(bw, n - 1 - k);
        for (uint32_t u = threadIdx.x; u < m; u += NT) {
            const double a = A[(size_t)(k + 1 + u) * bs + (u + 1)];
            ush[u] = a;
            lsh[u] = a / dk;
        }
        __syncthreads();
        const uint32_t ntri = m * (m + 1) / 2;
        for (uint32_t v = threadIdx.x; v < ntri; v += NT) {
            uint32_t ii = (uint32_t)((sqrt(8.0 * v + 1.0) - 1.0) * 0.5);
            while ((ii + 1) * (ii + 2) / 2 <= v) ++ii;  // exact triangular root
            while (ii * (ii + 1) / 2 > v) --ii;
            const uint32_t jj = v - ii * (ii + 1) / 2;
            A[(size_t)(k + 1 + ii) * bs + (ii - jj)] -= lsh[ii] * ush[jj];
        }
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < m; u += NT) A[(size_t)(k + 1 + u) * bs + (u + 1)] = lsh[u];
        __syncthreads();
    }
    // residual of the FP64 system in difference form, row order
    auto residual = [&](const double* xv, double* out_r, bool reordered) -> double {
        double part = 0.0;
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            const uint32_t g = base + i;
            const double xi = xv[i];
            double acc = e64[g] * xi;
            for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) acc += v64[k] * (xi - xv[col[k] - base]);
            if (chains) {
                const double a = gl64[i], c = gr64[i];
                if (a != 0.0) acc += a * (xi - xv[i - 1]);
                if (c != 0.0) acc += c * (xi - xv[i + 1]);
            }
            const double ri = bb[i] - acc;
            out_r[reordered ? perm[i] : i] = ri;
            part += ri * ri;
        }
        return sqrt(block_sum<NT>(part, sh));
    };
    double part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        rv[i] = bb[i];
        part += bb[i] * bb[i];
    }
    const double bn = sqrt(block_sum<NT>(part, sh));
    double rn = bn;
    int steps = 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (; steps < 12 && rn > 1e-16 * bn; ++steps) {
        for (uint32_t i = threadIdx.x; i < n; i += NT) t[perm[i]] = rv[i];
        __syncthreads();
        if (warp == 0) {
            for (uint32_t k = 0; k < n; ++k) {  // forward: t_i -= l_ik t_k
                const double tk = t[k];
                const uint32_t m = min(bw, n - 1 - k);
                for (uint32_t u = lane; u < m; u += 32) t[k + 1 + u] -= A[(size_t)(k + 1 + u) * bs + (u + 1)] * tk;
                __syncwarp();
            }
            for (uint32_t k = lane; k < n; k += 32) t[k] /= A[(size_t)k * bs];
            __syncwarp();
            for (uint32_t kk = n; kk-- > 0;) {  // backward: t_k -= sum_i l_ik t_i
                const uint32_t m = min(bw, n - 1 - kk);
                double acc = 0.0;
                for (uint32_t u = lane; u < m; u += 32) acc += A[(size_t)(kk + 1 + u) * bs + (u + 1)] * t[kk + 1 + u];
#pragma unroll
                for (int s2 = 16; s2 > 0; s2 >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s2);
                if (lane == 0) t[kk] -= acc;
                __syncwarp();
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += NT) xt[i] = xx[i] + t[perm[i]];
        __syncthreads();
        const double rn_new = residual(xt, t, true);  // t is free again: it holds the candidate residual
        if (!(rn_new < rn)) { ++steps; break; }  // at the rounding floor
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            xx[i] = xt[i];
            rv[i] = t[perm[i]];
        }
        __syncthreads();
        rn = rn_new;
        if (rn <= tol * bn * 1e-3) { ++steps; break; }
    }
    part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) part += bb[i] * (1.0 - xx[i]);
    const double G = block_sum<NT>(part, sh);
    if (threadIdx.x == 0) {
        o.G = G;
        o.res = bn > 0 ? rn / bn : 0.0;
        o.outer = steps;
        o.inner = 0;
        out[rr] = o;
    }
}

// Narrow bands (b <= kDcWin): the same factorisation with the b + 1 active
// rows in a shared-memory window (row i in slot i mod (b + 1)), the next row
// fetched while the current pivot updates, L written by columns
// (Lc[k b + u] = l_{k+1+u,k}) and the pivots to D, so the substitutions read
// one contiguous column per step; the solve vector lives in shared memory when
// it fits (n <= kDcShN). T is the type of the factors and of the correction
// solves: float by default (a GB300 SM issues FP64 at a small fraction of its
// FP32 rate, and one CTA factors sequentially), double when refinement with
// FP32 factors stalls above the tolerance (condition number near 1 / eps32).
// The residual and x stay in FP64 either way; each correction solves for the
// residual scaled to unit norm.
constexpr uint32_t kDcWin = 64;
constexpr uint32_t kDcShN = 12288;

template <int NT, typename T>
__global__ void __launch_bounds__(NT) k_dc_band_win(int R, const uint32_t* __restrict__ abase,
                                                    const unsigned long long* __restrict__ boff,
                                                    const uint32_t* __restrict__ bwid,
                                                    const uint32_t* __restrict__ permL,
                                                    const uint32_t* __restrict__ rowp, const uint32_t* __restrict__ col,
                                                    const double* __restrict__ v64, const double* __restrict__ e64,
                                                    const double* __restrict__ ch64, int chains,
                                                    const double* __restrict__ b, double* __restrict__ x,
                                                    double* __restrict__ r64, double* __restrict__ band,
                                                    double* __restrict__ work, double tol, int tshared,
                                                    CgOut* __restrict__ out) {
    __shared__ double sh[96];
    __shared__ T win[(kDcWin + 1) * (kDcWin + 1)];
    __shared__ T lsh[kDcWin], ush[kDcWin];
    extern __shared__ __align__(8) unsigned char tsh_raw[];
    T* tsh = reinterpret_cast<T*>(tsh_raw);
    const int rr = blockIdx.x;
    if (rr >= R) return;
    const uint32_t base = abase[rr], n = abase[rr + 1] - base, bw = bwid[rr], bs = bw + 1;
    CgOut o{};
    o.n = (int)n;
    if (n == 0) {
        if (threadIdx.x == 0) out[rr] = o;
        return;
    }
    // band rows (n x bs), then L by columns (n x bw), then D (n)
    double* A = band + boff[rr] * 2;  // rows (n bs) + L (n bw) + D (n) = 2 n bs
    T* Lc = reinterpret_cast<T*>(A + (size_t)n * bs);
    T* D = Lc + (size_t)n * bw;
    const uint32_t* perm = permL + base;
    const double* bb = b + base;
    double* xx = x + base;
    double* rv = r64 + base;
    T* tg = reinterpret_cast<T*>(work + base);  // solve vector in global memory (large n)
    double* xt = work + abase[R] + base;        // candidate x
    double* rc = r64 + abase[R] + base;         // candidate residual, reordered
    T* t = tshared ? tsh : tg;  // the launch sized tsh for every realisation
    const double* gl64 = ch64 + base;
    const double* gr64 = ch64 + abase[R] + base;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        const uint32_t g = base + i, p = perm[i];
        double* row = A + (size_t)p * bs;
        for (uint32_t q = 1; q < bs; ++q) row[q] = 0.0;
        double d = e64[g];
        for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) {
            d += v64[k];
            const uint32_t q = perm[col[k] - base];
            if (q < p && p - q <= bw) row[p - q] -= v64[k];
        }
        if (chains) {
            if (gl64[i] > 0.0) {
                d += gl64[i];
                const uint32_t q = perm[i - 1];
                if (q < p && p - q <= bw) row[p - q] -= gl64[i];
            }
            if (gr64[i] > 0.0) {
                d += gr64[i];
                const uint32_t q = perm[i + 1];
                if (q < p && p - q <= bw) row[p - q] -= gr64[i];
            }
        }
        row[0] = d;
        xx[i] = 0.0;
    }
    __syncthreads();
    const uint32_t w0 = min(bs, n);  // rows 0..b into the window
    for (uint32_t e = threadIdx.x; e < w0 * bs; e += NT) win[e] = (T)A[e];
    // row k + bs enters slot k % bs after pivot k; it is fetched one pivot
    // ahead so that its load overlaps a whole pivot
    T pre = 0;
    if (bs < n && threadIdx.x < bs) pre = (T)A[(size_t)bs * bs + threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t sk = 0;  // slot of row k
    if (bw < 32) {
        // one warp, no block barriers: lane ii owns trailing row k + 1 + ii and
        // receives the pivot column's entries by shuffle; rows enter the window
        // from a 4-deep register ring (row k + bs + j fetched four pivots early)
        if (warp == 0) {
            (void)pre;
            T ring[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                ring[j] = (bs + j < n && (uint32_t)lane < bs) ? (T)A[(size_t)(bs + j) * bs + lane] : (T)0;
            for (uint32_t k0 = 0; k0 < n; k0 += 4) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t k = k0 + j;
                    if (k < n) {
                        const uint32_t m = min(bw, n - 1 - k);
                        const T dk = win[sk * bs];
                        uint32_t sl = sk + 1 + lane;
                        sl -= sl >= bs ? bs : 0;
                        T a = 0, l = 0;
                        if ((uint32_t)lane < m) {
                            a = win[sl * bs + lane + 1];
                            l = a / dk;
                        }
#pragma unroll 4
                        for (uint32_t jj = 0; jj < m; ++jj) {
                            const T u = __shfl_sync(0xffffffffu, a, jj);
                            if ((uint32_t)lane < m && jj <= (uint32_t)lane) win[sl * bs + (lane - jj)] -= l * u;
                        }
                        if ((uint32_t)lane < m) {
                            win[sl * bs + lane + 1] = l;
                            Lc[(size_t)k * bw + lane] = l;
                        }
                        if (lane == 0) D[k] = dk;
                        __syncwarp();
                        if (k + bs < n && (uint32_t)lane < bs) win[sk * bs + lane] = ring[j];
                        const uint32_t nr = k + bs + 4;
                        ring[j] = (nr < n && (uint32_t)lane < bs) ? (T)A[(size_t)nr * bs + lane] : (T)0;
                        sk = sk + 1 == bs ? 0 : sk + 1;
                        __syncwarp();
                    }
                }
            }
        }
        __syncthreads();
    } else
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t m = min(bw, n - 1 - k);
        const T dk = win[sk * bs];
        T pre2 = 0;
        if (k + 1 + bs < n && threadIdx.x < bs) pre2 = (T)A[(size_t)(k + 1 + bs) * bs + threadIdx.x];
        for (uint32_t u = threadIdx.x; u < m; u += NT) {
            uint32_t sl = sk + 1 + u;
            sl -= sl >= bs ? bs : 0;
            const T a = win[sl * bs + (u + 1)];
            ush[u] = a;
            lsh[u] = a / dk;
        }
        __syncthreads();
        // trailing triangle, (ii, jj) from a power-of-two split of the index
        const uint32_t lg = m > 1 ? 32 - __clz(m - 1) : 0;
        for (uint32_t v = threadIdx.x; v < (m << lg); v += NT) {
            const uint32_t ii = v >> lg, jj = v & ((1u << lg) - 1u);
            if (jj <= ii) {
                uint32_t sl = sk + 1 + ii;
                sl -= sl >= bs ? bs : 0;
                win[sl * bs + (ii - jj)] -= lsh[ii] * ush[jj];
            }
        }
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < m; u += NT) {
            uint32_t sl = sk + 1 + u;
            sl -= sl >= bs ? bs : 0;
            win[sl * bs + (u + 1)] = lsh[u];
            Lc[(size_t)k * bw + u] = lsh[u];
        }
        if (threadIdx.x == 0) D[k] = dk;
        if (k + bs < n && threadIdx.x < bs) win[sk * bs + threadIdx.x] = pre;
        pre = pre2;
        sk = sk + 1 == bs ? 0 : sk + 1;
        __syncthreads();
    }
    auto residual = [&](const double* xv, bool reordered) -> double {
        double part = 0.0;
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            const uint32_t g = base + i;
            const double xi = xv[i];
            double acc = e64[g] * xi;
            for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) acc += v64[k] * (xi - xv[col[k] - base]);
            if (chains) {
                const double a = gl64[i], c = gr64[i];
                if (a != 0.0) acc += a * (xi - xv[i - 1]);
                if (c != 0.0) acc += c * (xi - xv[i + 1]);
            }
            const double ri = bb[i] - acc;
            if (reordered) rc[i] = ri; else rv[i] = ri;
            part += ri * ri;
        }
        return sqrt(block_sum<NT>(part, sh));
    };
    double part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        rv[i] = bb[i];
        part += bb[i] * bb[i];
    }
    const double bn = sqrt(block_sum<NT>(part, sh));
    double rn = bn;
    int steps = 0;
    const int max_steps = sizeof(T) == 4 ? 40 : 12;
    for (; steps < max_steps && rn > 1e-16 * bn; ++steps) {
        const double sc = 1.0 / rn;
        for (uint32_t i = threadIdx.x; i < n; i += NT) t[perm[i]] = (T)(rv[i] * sc);
        __syncthreads();
        if (warp == 0 && bw < 32) {
            // blocks of 32 rows, lane j on row B + j. Forward: the rows' sums
            // over the columns of earlier blocks (all loads issued first), then
            // the block's own triangle through shuffles: t_c final, the rows
            // below it lose l_{jc} t_c.
            for (uint32_t B = 0; B < n; B += 32) {
                const uint32_t i = B + lane;
                const bool on = i < n;
                T acc = on ? t[i] : (T)0;
                {
                    T lv[32], tv[32];
#pragma unroll
                    for (int kk = 0; kk < 32; ++kk) {
                        const bool ok = on && (uint32_t)kk < bw && B + kk >= bw;
                        const uint32_t k = ok ? B + kk - bw : 0;
                        const bool in = ok && i - k <= bw;
                        lv[kk] = in ? Lc[(size_t)k * bw + (i - k - 1)] : (T)0;
                        tv[kk] = in ? t[k] : (T)0;
                    }
#pragma unroll
                    for (int kk = 0; kk < 32; ++kk) acc -= lv[kk] * tv[kk];
                }
                T lr[32];
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    const uint32_t kc = B + c;
                    lr[c] = (on && c < lane && (uint32_t)(lane - c) <= bw && kc < n)
                                ? Lc[(size_t)kc * bw + (lane - c - 1)] : (T)0;
                }
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    const T tc = __shfl_sync(0xffffffffu, acc, c);
                    if (c < lane) acc -= lr[c] * tc;
                }
                if (on) t[i] = acc;
                __syncwarp();
            }
            for (uint32_t k = lane; k < n; k += 32) t[k] /= D[k];
            __syncwarp();
            // backward, blocks from the last: the rows' sums over the rows of
            // later blocks (their own columns, contiguous), then the block's
            // triangle from its last row up
            const uint32_t nb = (n + 31) / 32;
            for (uint32_t bi = nb; bi-- > 0;) {
                const uint32_t B = bi * 32, k = B + lane;
                const bool on = k < n;
                T acc = on ? t[k] : (T)0;
                const uint32_t top = B + 32;  // first row of the next block
                {
                    T lv[32], tv[32];
#pragma unroll
                    for (int u = 0; u < 32; ++u) {
                        const uint32_t r = k + 1 + u;
                        const bool in = on && (uint32_t)u < bw && r >= top && r < n;
                        lv[u] = in ? Lc[(size_t)k * bw + u] : (T)0;
                        tv[u] = in ? t[r] : (T)0;
                    }
#pragma unroll
                    for (int u = 0; u < 32; ++u) acc -= lv[u] * tv[u];
                }
                T lr[32];
#pragma unroll
                for (int c = 0; c < 32; ++c) {
                    lr[c] = (on && c > lane && (uint32_t)(c - lane) <= bw && B + c < n)
                                ? Lc[(size_t)k * bw + (c - lane - 1)] : (T)0;
                }
#pragma unroll
                for (int c = 31; c >= 0; --c) {
                    const T tc = __shfl_sync(0xffffffffu, acc, c);
                    if (c > lane) acc -= lr[c] * tc;
                }
                if (on) t[k] = acc;
                __syncwarp();
            }
        } else if (warp == 0) {
            // forward: t_{k+1+u} -= l_{k+1+u,k} t_k; the columns come from an
            // 8-deep register ring, each fetched 8 steps before its use
            constexpr int P = 8;
            T r0[P], r1[P];
            auto col_of = [&](uint32_t k, T* a0, T* a1) {
                *a0 = 0;
                *a1 = 0;
                if (k < n) {
                    const uint32_t m = min(bw, n - 1 - k);
                    if ((uint32_t)lane < m) *a0 = Lc[(size_t)k * bw + lane];
                    if ((uint32_t)lane + 32 < m) *a1 = Lc[(size_t)k * bw + lane + 32];
                }
            };
#pragma unroll
            for (int j = 0; j < P; ++j) col_of((uint32_t)j, &r0[j], &r1[j]);
            for (uint32_t k0 = 0; k0 < n; k0 += P) {
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    const uint32_t k = k0 + j;
                    if (k < n) {
                        const uint32_t m = min(bw, n - 1 - k);
                        const T tk = t[k];
                        if ((uint32_t)lane < m) t[k + 1 + lane] -= r0[j] * tk;
                        if ((uint32_t)lane + 32 < m) t[k + 33 + lane] -= r1[j] * tk;
                        col_of(k + P, &r0[j], &r1[j]);
                    }
                    __syncwarp();
                }
            }
            for (uint32_t k = lane; k < n; k += 32) t[k] /= D[k];
            __syncwarp();
            // backward: t_k -= sum_u l_{k+1+u,k} t_{k+1+u}, columns from the ring
#pragma unroll
            for (int j = 0; j < P; ++j) col_of(n - 1 - (uint32_t)j < n ? n - 1 - (uint32_t)j : n, &r0[j], &r1[j]);
            for (uint32_t k0 = 0; k0 < n; k0 += P) {
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    const uint32_t step = k0 + j;
                    if (step < n) {
                        const uint32_t kk = n - 1 - step;
                        const uint32_t m = min(bw, n - 1 - kk);
                        T acc = 0;
                        if ((uint32_t)lane < m) acc = r0[j] * t[kk + 1 + lane];
                        if ((uint32_t)lane + 32 < m) acc += r1[j] * t[kk + 33 + lane];
#pragma unroll
                        for (int s2 = 16; s2 > 0; s2 >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s2);
                        if (lane == 0) t[kk] -= acc;
                        col_of(step + P < n ? n - 1 - (step + P) : n, &r0[j], &r1[j]);
                    }
                    __syncwarp();
                }
            }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += NT) xt[i] = xx[i] + rn * (double)t[perm[i]];
        __syncthreads();
        const double rn_new = residual(xt, true);
        if (!(rn_new < rn)) { ++steps; break; }  // at the rounding floor
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            xx[i] = xt[i];
            rv[i] = rc[i];
        }
        __syncthreads();
        rn = rn_new;
        if (rn <= tol * bn * 1e-3) { ++steps; break; }
    }
    part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) part += bb[i] * (1.0 - xx[i]);
    const double G = block_sum<NT>(part, sh);
    if (threadIdx.x == 0) {
        o.G = G;
        o.res = bn > 0 ? rn / bn : 0.0;
        o.outer = steps;
        o.inner = 0;
        out[rr] = o;
    }
}

// Direct form for bands of at most 32 (the rod and node networks of the
// jammed box: 28 and 30): block cyclic reduction (nf_bcr.cuh) in one CTA per
// realisation, then the same FP64 refinement as the banded forms. The blocks
// are assembled straight from the CSR rows in band order (row p of the band
// is block p / 32, row p mod 32); the rows past n pad the last block with an
// identity. Factors in T (float first, double when float stalls above the
// tolerance); x and the residual stay in FP64.
template <int NT, typename T>
__global__ void __launch_bounds__(NT) k_dc_bcr(int R, const uint32_t* __restrict__ abase,
                                               const uint32_t* __restrict__ boff, const uint32_t* __restrict__ permL,
                                               const uint32_t* __restrict__ rowp, const uint32_t* __restrict__ col,
                                               const double* __restrict__ v64, const double* __restrict__ e64,
                                               const double* __restrict__ ch64, int chains,
                                               const double* __restrict__ b, double* __restrict__ x,
                                               double* __restrict__ r64, T* __restrict__ blocks,
                                               T* __restrict__ tvec, double* __restrict__ work, double tol,
                                               int retry, CgOut* __restrict__ out) {
    __shared__ double sh[96];
    __shared__ int bad;
    extern __shared__ __align__(16) unsigned char bcr_sh[];
    T* S = reinterpret_cast<T*>(bcr_sh) + (threadIdx.x >> 5) * kBcrScratch;  // this warp's scratch
    const int rr = blockIdx.x;
    if (rr >= R) return;
    if (retry && (out[rr].n == 0 || out[rr].res <= tol)) return;  // solved by the previous pass
    const uint32_t base = abase[rr], n = abase[rr + 1] - base;
    CgOut o{};
    o.n = (int)n;
    if (n == 0) {
        if (threadIdx.x == 0) out[rr] = o;
        return;
    }
    const uint32_t m = boff[rr + 1] - boff[rr];
    T* blk = blocks + (size_t)boff[rr] * kBcrPer;
    T* t = tvec + (size_t)boff[rr] * kBcrW;
    const uint32_t* perm = permL + base;
    const double* bb = b + base;
    double* xx = x + base;
    double* rv = r64 + base;
    double* xt = work + base;            // candidate x
    double* rc = r64 + abase[R] + base;  // candidate residual
    const double* gl64 = ch64 + base;
    const double* gr64 = ch64 + abase[R] + base;
    for (size_t e = threadIdx.x; e < (size_t)m * 2 * kBcrBlk; e += NT)
        blk[(e / (2 * kBcrBlk)) * kBcrPer + e % (2 * kBcrBlk)] = T(0);  // D and K of every block
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        const uint32_t g = base + i, p = perm[i], I = p >> 5;
        T* drow = blk + (size_t)I * kBcrPer + (p & 31u) * 32;
        T* krow = drow + kBcrBlk;
        auto put = [&](uint32_t q, double v) {
            const uint32_t J = q >> 5;
            if (J == I) drow[q & 31u] -= (T)v;
            else if (J + 1 == I) krow[q & 31u] -= (T)v;  // J == I + 1: the row of q writes it
        };
        double d = e64[g];
        for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) {
            d += v64[k];
            put(perm[col[k] - base], v64[k]);
        }
        if (chains) {
            if (gl64[i] > 0.0) {
                d += gl64[i];
                put(perm[i - 1], gl64[i]);
            }
            if (gr64[i] > 0.0) {
                d += gr64[i];
                put(perm[i + 1], gr64[i]);
            }
        }
        drow[p & 31u] += (T)d;
        xx[i] = 0.0;
    }
    for (uint32_t p = n + threadIdx.x; p < m * kBcrW; p += NT)
        blk[(size_t)(p >> 5) * kBcrPer + (p & 31u) * 33] = T(1);
    __syncthreads();
    const bool ok = bcr_factor<NT, T>(blk, m, S, &bad);
    double part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) {
        rv[i] = bb[i];
        part += bb[i] * bb[i];
    }
    const double bn = sqrt(block_sum<NT>(part, sh));
    double rn = bn;
    int steps = 0;
    const int max_steps = sizeof(T) == 4 ? 40 : 12;
    auto residual = [&](const double* xv) -> double {
        double acc2 = 0.0;
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            const uint32_t g = base + i;
            const double xi = xv[i];
            double acc = e64[g] * xi;
            for (uint32_t k = rowp[g], k1 = rowp[g + 1]; k < k1; ++k) acc += v64[k] * (xi - xv[col[k] - base]);
            if (chains) {
                const double a = gl64[i], c = gr64[i];
                if (a != 0.0) acc += a * (xi - xv[i - 1]);
                if (c != 0.0) acc += c * (xi - xv[i + 1]);
            }
            const double ri = bb[i] - acc;
            rc[i] = ri;
            acc2 += ri * ri;
        }
        return sqrt(block_sum<NT>(acc2, sh));
    };
    for (; ok && steps < max_steps && rn > 1e-16 * bn; ++steps) {
        const double sc = 1.0 / rn;
        for (uint32_t i = threadIdx.x; i < n; i += NT) t[perm[i]] = (T)(rv[i] * sc);
        for (uint32_t p = n + threadIdx.x; p < m * kBcrW; p += NT) t[p] = T(0);
        __syncthreads();
        bcr_solve<NT, T>(blk, m, t);
        for (uint32_t i = threadIdx.x; i < n; i += NT) xt[i] = xx[i] + rn * (double)t[perm[i]];
        __syncthreads();
        const double rn_new = residual(xt);
        if (!(rn_new < rn)) { ++steps; break; }  // at the rounding floor
        for (uint32_t i = threadIdx.x; i < n; i += NT) {
            xx[i] = xt[i];
            rv[i] = rc[i];
        }
        __syncthreads();
        const bool slow = rn_new > 1e-2 * rn;
        rn = rn_new;
        if (rn <= tol * bn * 1e-3) { ++steps; break; }
        // FP32 factors that gain fewer than two digits a step while still
        // above the tolerance would need tens of steps: the host refactors in
        // FP64 instead
        if (sizeof(T) == 4 && slow && rn > tol * bn) { ++steps; break; }
    }
    part = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += NT) part += bb[i] * (1.0 - xx[i]);
    const double G = block_sum<NT>(part, sh);
    if (threadIdx.x == 0) {
        o.G = G;
        o.res = !ok ? INFINITY : bn > 0 ? rn / bn : 0.0;
        o.outer = steps;
        o.inner = 0;
        out[rr] = o;
    }
}

nf_status Engine::solve_graph(uint32_t n, const std::vector<uint32_t>& off, const std::vector<uint32_t>& nodes,
                              uint32_t mc, uint32_t m, const uint32_t* eI, const uint32_t* eJ, const double* eG) {
    EventPair ev;
    NF_CK(ev.create());
    NF_CK(cudaEventRecord(ev.a, st));
    Asm A;
    nf_status s = assemble(n, off, mc, m, eI, eJ, eG, nullptr, &A);
    if (s != NF_OK) return s;
    const uint32_t nslot = n, na = A.na, nnz = A.nnz;
    uint32_t* act = eflag.p;
    uint32_t* errw = eflag.p + nslot + 1;
    NF_CK(volt.ensure(nslot + 1));
    NF_CK(xvec.ensure(na + 1));
    NF_CK(cgred.ensure(na + 1));
    NF_CK(cgbuf.ensure(5 * (size_t)na + 5));
    if (na)
        NF_LAUNCH(k_chain_factor, grid_for(na, 256), 256, 0, st)(na, chain64.p, chain64.p + na, cdiag.p, chain32.p);
    NF_CK(cudaGetLastError());
    // Host staging through the pinned buffer, 8-byte aligned regions:
    // active bases, the CSR rows for the ordering, the orders and block or
    // band offsets going back, the per-realisation results.
    size_t pofs = 0;
    auto region = [&](size_t bytes) {
        const size_t at = pofs;
        pofs = (pofs + bytes + 7) & ~size_t(7);
        return at;
    };
    const bool want_order = na > 0 && prm[0].solve_method != 2;
    const size_t p_ab = region(sizeof(uint32_t) * (R + 1));
    const size_t p_row = region(want_order ? sizeof(uint32_t) * (na + 1) : 0);
    const size_t p_col = region(want_order ? sizeof(uint32_t) * nnz : 0);
    const size_t p_gr = region(want_order ? sizeof(double) * na : 0);
    const size_t p_perm = region(want_order ? sizeof(uint32_t) * na : 0);
    const size_t p_bo = region(sizeof(uint32_t) * (R + 1));
    const size_t p_bw = region(sizeof(uint32_t) * R);
    const size_t p_hoff = region(sizeof(unsigned long long) * (R + 1));
    const size_t p_out = region(sizeof(CgOut) * R);
    s = ensure_pinned(pofs);
    if (s != NF_OK) return s;
    auto pin = [&](size_t at) { return hpin + at; };
    DBuf<uint32_t>& dab = rcur;  // per-realisation active base (R+1)
    NF_CK(dab.ensure(R + 1));
    std::memcpy(pin(p_ab), A.habase.data(), sizeof(uint32_t) * (R + 1));
    NF_CK(cudaMemcpyAsync(dab.p, pin(p_ab), sizeof(uint32_t) * (R + 1), cudaMemcpyHostToDevice, st));
    NF_CK(cgout.ensure(sizeof(CgOut) / sizeof(double) * (size_t)R + 1));
    CgOut* outs = reinterpret_cast<CgOut*>(cgout.p);
    const double tol = prm[0].solve_tol > 0 ? prm[0].solve_tol : 1e-10;
    const int max_inner = prm[0].solve_max_iter > 0 ? prm[0].solve_max_iter : 20000;
    // Direct form when every realisation's band after reverse Cuthill-McKee
    // is narrow: block cyclic reduction for bands up to 32 (SOLVE_METHOD 0 or
    // 1), else a banded LDL^T for bandwidth <= 512, n b^2 <= 1e9 updates, 1 GB
    // of band at most (SOLVE_METHOD 3 forces the banded form).
    const int method = prm[0].solve_method;
    bool direct = false, bcr = false;
    uint32_t bmax = 0;
    size_t nblk = 0;  // blocks of 32 unknowns over all realisations (block cyclic reduction)
    if (want_order) {
        uint32_t* hrow = reinterpret_cast<uint32_t*>(pin(p_row));
        uint32_t* hcol = reinterpret_cast<uint32_t*>(pin(p_col));
        double* hgr = reinterpret_cast<double*>(pin(p_gr));
        NF_CK(cudaMemcpyAsync(hrow, rowp.p, sizeof(uint32_t) * (na + 1), cudaMemcpyDeviceToHost, st));
        if (nnz) NF_CK(cudaMemcpyAsync(hcol, col.p, sizeof(uint32_t) * nnz, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(hgr, chain64.p + na, sizeof(double) * na, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        uint32_t* hperm = reinterpret_cast<uint32_t*>(pin(p_perm));
        uint32_t* hbo = reinterpret_cast<uint32_t*>(pin(p_bo));
        uint32_t* hbw = reinterpret_cast<uint32_t*>(pin(p_bw));
        unsigned long long* hoff = reinterpret_cast<unsigned long long*>(pin(p_hoff));
        hoff[0] = 0;
        bool fits = true, narrow = true;  // every band so far: banded form / block cyclic reduction
        int r = 0;
        std::vector<uint32_t> lrow, lcol, lp;
        std::vector<char> up;
        for (; r < R && (fits || narrow); ++r) {
            const uint32_t b0 = A.habase[r], nr = A.habase[r + 1] - b0;
            lrow.assign(nr + 1, 0);
            lcol.clear();
            up.assign(nr, 0);
            lcol.reserve(hrow[b0 + nr] - hrow[b0]);
            for (uint32_t i = 0; i < nr; ++i) {
                lrow[i] = (uint32_t)lcol.size();
                for (uint32_t k = hrow[b0 + i]; k < hrow[b0 + i + 1]; ++k) lcol.push_back(hcol[k] - b0);
                if (A.chains && i + 1 < nr) up[i] = hgr[b0 + i] > 0.0 ? 1 : 0;
            }
            lrow[nr] = (uint32_t)lcol.size();
            const uint32_t bw = nr ? rcm_order(nr, lrow, lcol, up, &lp) : 0;
            for (uint32_t i = 0; i < nr; ++i) hperm[b0 + i] = lp[i];
            hbw[r] = bw;
            bmax = std::max(bmax, bw);
            hoff[r + 1] = hoff[r] + (unsigned long long)nr * (bw + 1);  // rows; the window form adds L and D
            fits = fits && bw <= kDcBandMax && (double)nr * bw * bw <= 1e9;
            narrow = narrow && bw <= kBcrW;
        }
        const bool all = r == R;  // every realisation ordered
        hbo[0] = 0;
        for (int q = 0; q < R; ++q) hbo[q + 1] = hbo[q] + (A.habase[q + 1] - A.habase[q] + kBcrW - 1) / kBcrW;
        nblk = hbo[R];
        bcr = all && narrow && method != 3 && (double)nblk * (kBcrPer + kBcrW) * sizeof(double) <= 4e9;
        fits = bcr || (all && fits && (double)hoff[R] * sizeof(double) <= 1e9);
        if ((method == 1 || method == 3) && !fits) {
            err = "the reordered band is too wide for the direct form";
            return NF_ERR_PARAM;
        }
        direct = fits;
        if (direct) {
            NF_CK(dcperm.ensure(na));
            NF_CK(dcwork.ensure(2 * (size_t)na + 2));
            NF_CK(cudaMemcpyAsync(dcperm.p, hperm, sizeof(uint32_t) * na, cudaMemcpyHostToDevice, st));
            if (bcr) {
                NF_CK(bcrbuf.ensure(nblk * (kBcrPer + kBcrW)));
                NF_CK(bcroff.ensure(R + 1));
                NF_CK(cudaMemcpyAsync(bcroff.p, hbo, sizeof(uint32_t) * (R + 1), cudaMemcpyHostToDevice, st));
            } else {
                NF_CK(dcbw.ensure(R));
                NF_CK(dcboff.ensure(R + 1));
                NF_CK(dcband.ensure(2 * hoff[R] + na + 1));
                NF_CK(cudaMemcpyAsync(dcbw.p, hbw, sizeof(uint32_t) * R, cudaMemcpyHostToDevice, st));
                NF_CK(cudaMemcpyAsync(dcboff.p, hoff, sizeof(unsigned long long) * (R + 1), cudaMemcpyHostToDevice,
                                      st));
            }
        }
    }
    tstart(KT_CG);
    if (na == 0) {
        // every realisation's network is empty: G = 0, voltages from the components alone
    } else if (bcr) {
        NF_CK(cgred.ensure(2 * (size_t)na + 2));
        constexpr int kNtF = 384, kNtD = 256;  // registers: 170 a thread for float, 255 for double
        auto* kf32 = k_dc_bcr<kNtF, float>;
        auto* kf64 = k_dc_bcr<kNtD, double>;
        const int sh4 = (kNtF / 32) * kBcrScratch * (int)sizeof(float);
        const int sh8 = (kNtD / 32) * kBcrScratch * (int)sizeof(double);
        NF_CK(cudaFuncSetAttribute(kf32, cudaFuncAttributeMaxDynamicSharedMemorySize, sh4));
        NF_CK(cudaFuncSetAttribute(kf64, cudaFuncAttributeMaxDynamicSharedMemorySize, sh8));
        float* f32 = reinterpret_cast<float*>(bcrbuf.p);
        NF_LAUNCH(kf32, R, kNtF, sh4, st)(R, dab.p, bcroff.p, dcperm.p, rowp.p, col.p, val64.p, diag64.p, chain64.p,
                                          A.chains ? 1 : 0, bvec.p, xvec.p, cgred.p, f32, f32 + nblk * kBcrPer,
                                          dcwork.p, tol, 0, outs);
        NF_CK(cudaGetLastError());
        // FP64 factors for the realisations whose FP32 factors stayed above
        // the tolerance (the others return at once): no host round trip
        NF_LAUNCH(kf64, R, kNtD, sh8, st)(R, dab.p, bcroff.p, dcperm.p, rowp.p, col.p, val64.p, diag64.p,
                                          chain64.p, A.chains ? 1 : 0, bvec.p, xvec.p, cgred.p, bcrbuf.p,
                                          bcrbuf.p + nblk * kBcrPer, dcwork.p, tol, 1, outs);
    } else if (direct && bmax <= kDcWin) {
        uint32_t nmax = 0;
        for (int r = 0; r < R; ++r) nmax = std::max(nmax, A.habase[r + 1] - A.habase[r]);
        NF_CK(cgred.ensure(2 * (size_t)na + 2));
        const size_t sh4 = nmax <= kDcShN ? sizeof(float) * nmax : 0;
        auto* kf32 = k_dc_band_win<256, float>;
        auto* kf64 = k_dc_band_win<256, double>;
        NF_CK(cudaFuncSetAttribute(kf32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(float) * kDcShN)));
        NF_LAUNCH(kf32, R, 256, sh4, st)(R, dab.p, dcboff.p, dcbw.p, dcperm.p, rowp.p, col.p,
                                                             val64.p, diag64.p, chain64.p, A.chains ? 1 : 0, bvec.p,
                                                             xvec.p, cgred.p, dcband.p, dcwork.p, tol, sh4 ? 1 : 0,
                                                             outs);
        NF_CK(cudaGetLastError());
        const CgOut* h1 = reinterpret_cast<const CgOut*>(pin(p_out));
        NF_CK(cudaMemcpyAsync(pin(p_out), outs, sizeof(CgOut) * R, cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        bool again = false;
        for (int r = 0; r < R; ++r) again |= h1[r].n > 0 && !(h1[r].res <= tol);
        if (again) {  // FP32 factors too coarse for this system: FP64 factors
            const size_t sh8 = nmax <= kDcShN ? sizeof(double) * nmax : 0;
            NF_CK(cudaFuncSetAttribute(kf64, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(double) * kDcShN)));
            NF_LAUNCH(kf64, R, 256, sh8, st)(R, dab.p, dcboff.p, dcbw.p, dcperm.p, rowp.p, col.p,
                                                                  val64.p, diag64.p, chain64.p, A.chains ? 1 : 0,
                                                                  bvec.p, xvec.p, cgred.p, dcband.p, dcwork.p, tol,
                                                                  sh8 ? 1 : 0, outs);
        }
    } else if (direct) {
        NF_LAUNCH(k_dc_band<256>, R, 256, 0, st)(R, dab.p, dcboff.p, dcbw.p, dcperm.p, rowp.p, col.p, val64.p, diag64.p,
                                                chain64.p, A.chains ? 1 : 0, bvec.p, xvec.p, cgred.p, dcband.p,
                                                dcwork.p, tol, outs);
    } else {
        NF_LAUNCH(k_cg<512>, R, 512, 0, st)(R, dab.p, rowp.p, col.p, val32.p, val64.p, diag32.p, diag64.p, chain64.p,
                                     chain32.p, na, A.chains ? 1 : 0, bvec.p, xvec.p, cgred.p, cgbuf.p, tol, max_inner,
                                     outs);
    }
    NF_CK(cudaGetLastError());
    tstop(KT_CG);
    if (nslot)
        NF_LAUNCH(k_scatter_v, grid_for(nslot, 256), 256, 0, st)(nslot, act, aidx.p, xvec.p, parent.p, cflag.p, volt.p,
                                                                 errw);
    NF_CK(cudaGetLastError());
    const CgOut* ho = reinterpret_cast<const CgOut*>(pin(p_out));
    if (na) NF_CK(cudaMemcpyAsync(pin(p_out), outs, sizeof(CgOut) * R, cudaMemcpyDeviceToHost, st));
    else std::memset(pin(p_out), 0, sizeof(CgOut) * R);
    NF_CK(cudaEventRecord(ev.b, st));
    NF_CK(cudaEventSynchronize(ev.b));
    float ms = 0;
    NF_CK(cudaEventElapsedTime(&ms, ev.a, ev.b));
    {
        double it = 0, ot = 0;
        for (int r = 0; r < R; ++r) { it += ho[r].inner; ot += ho[r].outer; }
        tbytes(KT_CG, it * (8.0 * nnz + 24.0 * na) + ot * (12.0 * nnz + 40.0 * na), it * (2.0 * nnz + 10.0 * na));
    }
    solve_st.assign(R, nf_solve_stats{});
    bool conv = true;
    for (int r = 0; r < R; ++r) {
        nf_solve_stats& S = solve_st[r];
        S.G_eff = ho[r].G;
        S.residual = ho[r].res;
        S.outer_iters = ho[r].outer;
        S.inner_iters = ho[r].inner;
        S.n_nodes = nodes[r];
        S.n_active = A.habase[r + 1] - A.habase[r];
        S.percolating = S.n_active > 0;
        S.ms = ms;
        S.direct = bcr ? 2 : direct ? 1 : 0;
        S.bandwidth = direct ? bmax : 0;
        if (S.n_active > 0 && !(S.residual <= tol)) conv = false;
    }
    solve_valid = true;
    if (!conv) { err = "network solve did not reach its tolerance"; return NF_ERR_NOT_CONVERGED; }
    return NF_OK;
}

// ---------------------------------------------------------------------------
// Adjoint.
// ---------------------------------------------------------------------------
__global__ void k_adjoint(uint32_t lo, uint32_t hi, uint32_t rod0, const Real* __restrict__ reals, uint32_t r,
                          const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                          const double* __restrict__ t0, const double* __restrict__ t1, const double* __restrict__ D,
                          const double* __restrict__ G, const int8_t* __restrict__ img,
                          const float4* __restrict__ pos, const float4* __restrict__ dir,
                          const double* __restrict__ V, double* __restrict__ grad, double* __restrict__ acc) {
    uint32_t e = lo + blockIdx.x * blockDim.x + threadIdx.x;
    double dl = 0.0, dg0 = 0.0;
    if (e < hi) {
        const Real& Re = reals[r];
        const uint32_t i = I[e], j = J[e];
        const float4 pA = pos[i], cA = dir[i];
        double dv, gap;
        if (j == NF_SRC_ELEC) { dv = 1.0 - V[i]; gap = D[e] - cA.w; }
        else if (j == NF_SNK_ELEC) { dv = V[i]; gap = D[e] - cA.w; }
        else { dv = V[i] - V[j]; gap = D[e] - cA.w - dir[j].w; }
        const double w = dv * dv;
        dg0 = w * G[e] / Re.G0;
        const bool clamped = !(gap > Re.dc);
        if (!clamped) {
            dl = w * G[e] * (gap - Re.dc) / (Re.lambda * Re.lambda);
            const double dGdD = -G[e] / Re.lambda * w;
            const double uI = t0[e] / pA.w + 0.5;
            double* gi = grad + 6ull * (i - rod0);
            if (j >= NF_SNK_ELEC) {
                const int f = Re.field_axis;
                const double sg = (j == NF_SRC_ELEC) ? 1.0 : -1.0;
                atomicAdd(&gi[f], dGdD * sg * (1.0 - uI));
                atomicAdd(&gi[3 + f], dGdD * sg * uI);
            } else {
                const float4 pB = pos[j], cB = dir[j];
                const double sh[3] = {img[3 * e] * (double)Re.L[0], img[3 * e + 1] * (double)Re.L[1],
                                      img[3 * e + 2] * (double)Re.L[2]};
                const double pa[3] = {pA.x + t0[e] * cA.x, pA.y + t0[e] * cA.y, pA.z + t0[e] * cA.z};
                const double pb[3] = {(pB.x + sh[0]) + t1[e] * cB.x, (pB.y + sh[1]) + t1[e] * cB.y,
                                      (pB.z + sh[2]) + t1[e] * cB.z};
                const double uJ = t1[e] / pB.w + 0.5;
                double* gj = grad + 6ull * (j - rod0);
                for (int d = 0; d < 3; ++d) {
                    const double gd = (pa[d] - pb[d]) / D[e] * dGdD;
                    atomicAdd(&gi[d], gd * (1.0 - uI));
                    atomicAdd(&gi[3 + d], gd * uI);
                    atomicAdd(&gj[d], -gd * (1.0 - uJ));
                    atomicAdd(&gj[3 + d], -gd * uJ);
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        dl += __shfl_down_sync(0xffffffffu, dl, o);
        dg0 += __shfl_down_sync(0xffffffffu, dg0, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&acc[0], dl);
        atomicAdd(&acc[1], dg0);
    }
}

nf_status Engine::adjoint(int r, float* dG_dend, size_t cap, double* dlam, double* dg0) {
    if (!solve_valid) { err = "no solution: run nf_solve first"; return NF_ERR_STATE; }
    if (r < 0 || r >= R) return NF_ERR_PARAM;
    const uint32_t n = count[r];
    if (dG_dend && cap < (size_t)n) { err = "gradient buffer too small"; return NF_ERR_CAPACITY; }
    DBuf<double> g;
    NF_CK(g.ensure(6ull * n + 2));
    NF_CK(cudaMemsetAsync(g.p, 0, sizeof(double) * (6ull * n + 2), st));
    const uint32_t lo = (uint32_t)ct_off[r], hi = (uint32_t)ct_off[r + 1];
    if (hi > lo)
        NF_LAUNCH(k_adjoint, grid_for(hi - lo, 256), 256, 0, st)(lo, hi, hreal[r].rod_off, dreal.p, (uint32_t)r, cI.p, cJ.p,
                                                          ct0.p, ct1.p, cD.p, cG.p, cimg.p, pos.p, dir.p, volt.p, g.p,
                                                          g.p + 6ull * n);
    NF_CK(cudaGetLastError());
    std::vector<double> h(6ull * n + 2);
    NF_CK(cudaMemcpyAsync(h.data(), g.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    g.release();
    if (dG_dend)
        for (size_t k = 0; k < 6ull * n; ++k) dG_dend[k] = (float)h[k];
    if (dlam) *dlam = h[6ull * n];
    if (dg0) *dg0 = h[6ull * n + 1];
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
