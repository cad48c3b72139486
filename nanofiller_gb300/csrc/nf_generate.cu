// nf_generate.cu -- seeded candidate stream, von Neumann density test and
// cell-list hard-core rejection with sequential-insertion semantics.
//
// Reference path replaced: cudaMain / cudaGenStep (src/cudaMain.cu:61-161,
// :219-351) with cuda_CNTgenerate_orient (inc/cuda_CNTgenerate.h:136-260),
// cuda_InternalIsect_noLck, cuda_NewExtIsectLB_parted, cuda_OldExtIsectLB
// (inc/intersection_kern.h:12-364) and cuda_renewOcc (inc/auxilary_kernels.h:11-26).
//
// Semantics: candidate k (stream order) is accepted iff its density variate
// passes (u < rho(x)) and it hits no rod accepted before it; generation stops
// at the target count or when the stream budget is spent. Each round draws a
// block of stream indices per realisation and
//   1. recomputes candidates, keeps those passing the density test (scan),
//   2. bins them by cell (counting sort),
//   3. tests each against every accepted rod in the 27 neighbour cells,
//   4. records, for survivors, the earlier survivors of the same round they hit,
//   5. resolves those in stream order (a candidate is rejected once an earlier
//      neighbour is accepted and accepted once all earlier neighbours are
//      rejected; monotone, so passes converge to the sequential answer),
//   6. appends the accepted in stream order up to the target.
// The reference instead kills a same-cell candidate on conflict with any later
// candidate (inc/intersection_kern.h:69-72) and lets parity scheduling decide
// cross-cell conflicts (:119-126); its result depends on launch order.
#include <algorithm>
#include <cmath>
#include <cstring>

#include <cub/device/device_scan.cuh>

#include "nf_engine.cuh"
#include "nf_tiles.cuh"

namespace nf {

// ---------------------------------------------------------------------------
// Host-side derived parameters (same arithmetic as the oracle).
// ---------------------------------------------------------------------------
int64_t target_count(const nf_params& p) {
    if (p.n_target > 0) return p.n_target;
    double V = (double)p.box[0] * p.box[1] * p.box[2];
    double El = p.l, Ea2 = (double)p.a * p.a;
    if (p.len_mode == NF_SIZE_LOGNORMAL) {
        double s = 0, w = 0;
        for (int i = -6000; i <= 6000; ++i) {
            double z = i * 1e-3, g = std::exp(-0.5 * z * z);
            double v = p.l * std::exp(p.len_sigma_ln * z);
            v = std::min(std::max(v, (double)p.len_min), (double)p.len_max);
            s += g * v;
            w += g;
        }
        El = s / w;
    }
    if (p.rad_mode == NF_SIZE_UNIFORM) {
        double lo = p.rad_min, hi = p.rad_max;
        Ea2 = (hi * hi + hi * lo + lo * lo) / 3.0;
    }
    double vinc = M_PI * Ea2 * El;
    return (int64_t)std::ceil((double)p.vf * V / vinc);
}

static void size_bounds(const nf_params& p, double* lmax, double* amax) {
    *lmax = (p.len_mode == NF_SIZE_LOGNORMAL) ? (double)p.len_max : (double)p.l;
    *amax = (p.rad_mode == NF_SIZE_UNIFORM) ? (double)std::max(p.rad_min, p.rad_max) : (double)p.a;
}

// One cell grid serves all stages: its edge covers the widest pair reach of
// the hard-core test, the contact test and the screening test.
double stage_reach(const nf_params& p) {
    double lmax, amax;
    size_bounds(p, &lmax, &amax);
    double eps = p.tol, epc = (double)1e-6f;
    double h = lmax / 2 + amax + std::max(eps, epc);
    double gen = 2 * h + ((2 * amax) * p.sc_frac + p.sep + eps);
    double con = 2 * h + (2 * amax + p.stat_dist_lim + epc);
    return std::max(gen, con);
}

// The reference's angle law (genCosine / sym_truncNormal,
// inc/cuda_CNTgenerate.h:262-275): theta (from the preferred axis) normal about
// DEF_THETA_MED truncated to +- pi/2, phi about DEF_PHI_MED truncated to +- pi,
// each only where its deviation is positive; the constants of tn_angle.
void tn_consts(float s, double w, int ref, double* c1, double* c2, double* zmax) {
    const double sd = (double)s;
    const double z = ddiv(ddiv(w, sd), kSqrt2);
    if (ref) {
        *c1 = dmul(0.5, erf_d(z));
        *c2 = dmul(dmul(2.0, sd), kSqrt2);
        *zmax = 1e300;
    } else {
        *c1 = erf_d(z);
        *c2 = dmul(sd, kSqrt2);
        *zmax = z;
    }
}

void set_tn_law(Real& R, const nf_params& p) {
    R.tn = (p.theta_dev > 0 ? 1 : 0) | (p.phi_dev > 0 ? 2 : 0);
    R.tmed = p.theta_med;
    R.pmed = p.phi_med;
    if (R.tn & 1) tn_consts(p.theta_dev, dmul(kPiD, 0.5), p.ref_trunc_normal, &R.tc1, &R.tc2, &R.tz);
    if (R.tn & 2) tn_consts(p.phi_dev, kPiD, p.ref_trunc_normal, &R.pc1, &R.pc2, &R.pz);
}

// Tube grid of the pair sweeps (nf_tube.cuh). The registration radius is half
// the widest pair threshold of the three sweeps (hard core, contacts,
// screening) with margins far above the FP32 rounding of the walk; the cell
// edge e solves n (2 l e^2 + e^3) = load, the registrations per cell of n rods
// per unit volume of mean length l (each registers in ~2 l / e + 1 cells of
// volume e^3), capped so that along a periodic axis a dilated segment spans
// less than the box edge minus two cells; where no cell of at least 4 trho
// allows that, the stencil sweeps run.
void set_tube_grid(Real& R, const nf_params& p) {
    R.tube = 0;
    if (p.tube_load < 0) return;
    double lmax, amax;
    size_bounds(p, &lmax, &amax);
    const double eps = std::max((double)p.tol, (double)1e-6f);
    const double thr = std::max(2 * amax * p.sc_frac + p.sep + eps, 2 * amax + p.stat_dist_lim + eps);
    const double Lmax = std::max((double)p.box[0], std::max((double)p.box[1], (double)p.box[2]));
    const double rho = 0.5 * thr * 1.0001 + 1e-5 * (1.0 + Lmax) + 8.0 * R.slack;
    const double h = (lmax / 2 + amax + eps) * 1.00001 + R.slack;
    const int per = (R.per_gen | R.per_con) & 7, per_both = R.per_gen & R.per_con & 7;
    const double V = (double)p.box[0] * p.box[1] * p.box[2];
    const double nrod = (double)std::max<int64_t>(target_count(p), 1);
    double lmean = p.l;
    if (p.len_mode == NF_SIZE_LOGNORMAL) lmean = std::min((double)p.len_max, p.l * std::exp(0.5 * p.len_sigma_ln * p.len_sigma_ln));
    const double load = p.tube_load > 0 ? (double)p.tube_load : 64.0;
    const double nd = nrod / V;
    double lo = 4 * rho, hi = std::max(lo, std::min((double)p.box[0], std::min((double)p.box[1], (double)p.box[2])));
    for (int it = 0; it < 60; ++it) {
        const double e = 0.5 * (lo + hi);
        if (nd * (2 * lmean * e * e + e * e * e) > load) hi = e; else lo = e;
    }
    double e = std::max(0.5 * (lo + hi), 4 * rho);
    // along a periodic axis a dilated segment must span less than the box
    // edge minus two cells, so that an object reaches a cell through one copy
    // only (one image away at most)
    for (int d = 0; d < 3; ++d)
        if ((per >> d) & 1) e = std::min(e, 0.5 * (0.999 * p.box[d] - 2 * (h + rho)));
    if (!(e >= 4 * rho)) return;
    for (;;) {
        uint64_t cells = 1;
        for (int d = 0; d < 3; ++d) {
            int n = (int)std::floor((double)p.box[d] / e);
            n = n < 1 ? 1 : n;
            // one copy per cell along a periodic axis (finer cells where the edge rounded up)
            while (((per >> d) & 1) && !(2 * (h + rho) < 0.999 * p.box[d] - 2.0 * p.box[d] / n) && n < (1 << 20)) ++n;
            R.tcn[d] = n;
            R.tce[d] = (float)((double)p.box[d] / R.tcn[d]);
            R.tci[d] = (float)((double)R.tcn[d] / (double)p.box[d]);
            // margin cells beyond both faces of an axis open in some stage (an
            // object near an open face reaches past it)
            R.tcm[d] = ((per_both >> d) & 1) ? 0 : (int)std::ceil((h + rho) / R.tce[d]) + 1;
            cells *= (uint64_t)(R.tcn[d] + 2 * R.tcm[d]);
        }
        if (cells <= (1ull << 26)) { R.tncell = (uint32_t)cells; break; }
        e *= 1.25;
    }
    for (int d = 0; d < 3; ++d)
        if (((per >> d) & 1) && !(2 * (h + rho) < 0.999 * p.box[d] - 2.0 * R.tce[d])) return;
    R.trho = (float)rho;
    R.tube = 1;
}

Real make_real(const nf_params& p, const float* dmesh, int mn[3], double reach) {
    Real R;
    std::memset(&R, 0, sizeof(R));
    for (int d = 0; d < 3; ++d) R.L[d] = p.box[d];
    R.key[0] = (uint32_t)(p.seed & 0xffffffffu);
    R.key[1] = (uint32_t)(p.seed >> 32);
    R.orient = p.orient_mode;
    R.len_mode = p.len_mode;
    R.rad_mode = p.rad_mode;
    R.kappa = p.vmf_kappa;
    R.E2 = (p.orient_mode == NF_ORIENT_VMF) ? exp_nf(fmul(-2.0f, p.vmf_kappa)) : 0.0f;
    R.rot = (p.pref_ort[0] != 0.0f) || (p.pref_ort[1] != 0.0f);
    float cM, sM, cX, sX;
    sincos_turns((float)((double)p.pref_ort[0] / (2.0 * 3.14159265358979323846)), &cM, &sM);
    sincos_turns((float)((double)(-p.pref_ort[1]) / (2.0 * 3.14159265358979323846)), &cX, &sX);
    // inc_rotation (inc/cuda_CNTgenerate.h:289-295), Mu = phi, Xi = -theta
    R.m[0] = fmul(cM, cX);  R.m[1] = sM;   R.m[2] = fmul(-sX, cM);
    R.m[3] = fmul(-sM, cX); R.m[4] = cM;   R.m[5] = fmul(sX, sM);
    R.m[6] = sX;            R.m[7] = 0.0f; R.m[8] = cX;
    set_tn_law(R, p);
    R.l = p.l;
    R.a = p.a;
    R.sigma = p.len_sigma_ln;
    R.lmin = p.len_min;
    R.lmax = p.len_max;
    R.rmin = p.rad_min;
    R.rmax = p.rad_max;
    R.mesh = dmesh;
    for (int d = 0; d < 3; ++d) R.mn[d] = dmesh ? mn[d] : 0;
    R.dflt = p.density_default;
    R.per_gen = p.gen_periodic & 7;
    // contacts: the field axis is open with plane electrodes, periodic with
    // buffer-layer electrodes (their rods are the images beyond each face)
    R.per_con = (p.elec_buffer ? (p.gen_periodic | p.field_dir) : (p.gen_periodic & ~p.field_dir)) & 7;
    R.ebuf = p.elec_buffer && p.field_dir ? 1 : 0;
    // Cells of edge >= reach / S with a stencil of radius S. S = 2 tests about
    // 125 (reach/2)^3 of volume per probe instead of 27 reach^3 for S = 1; a
    // periodic axis needs at least S cells so that images stay within +-1.
    auto grid = [&](int S) {
        const double e = std::max(reach * 1.0001 / S, (double)p.cell_edge);
        double emin = 1e300;
        for (int d = 0; d < 3; ++d) {
            int c = (int)std::floor((double)p.box[d] / e);
            R.n[d] = c < 1 ? 1 : c;
            R.invE[d] = (float)((double)R.n[d] / (double)p.box[d]);
            emin = std::min(emin, (double)p.box[d] / R.n[d]);
        }
        R.S = std::max(1, (int)std::ceil(reach * 1.0001 / emin - 1e-9));
        for (int d = 0; d < 3; ++d)
            if (((R.per_gen | R.per_con) >> d & 1) && R.n[d] < R.S) return false;
        return R.S <= kStencilMax;
    };
    if (p.stencil_radius == 1 || !grid(2)) grid(1);
    R.eps = p.tol;
    R.scf = p.sc_frac;
    R.sep = p.sep;
    R.cut = p.stat_dist_lim;
    R.typo = p.ref_parallel_typo;
    float Lmax = std::max(p.box[0], std::max(p.box[1], p.box[2]));
    R.slack = Lmax * 9.5367431640625e-07f;  // 2^-20 L: coordinate rounding
    R.field_axis = p.field_dir == 1 ? 0 : (p.field_dir == 2 ? 1 : (p.field_dir == 4 ? 2 : -1));
    R.G0 = p.G0;
    R.lambda = p.lambda;
    R.dc = p.d_c;
    set_tube_grid(R, p);
    return R;
}

// ---------------------------------------------------------------------------
// Kernels.
// ---------------------------------------------------------------------------
// Density test of every stream slot of the round.
__global__ void k_stream_keep(const Real* __restrict__ reals, int R, const uint32_t* __restrict__ coff,
                              const uint64_t* __restrict__ kbeg, uint32_t nslots, uint32_t* __restrict__ keep) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    int r = find_real(coff, R, s);
    const Real& Re = reals[r];
    uint64_t k = kbeg[r] + (s - coff[r]);
    float4 p, d;
    float u, rho;
    candidate(Re, k, &p, &d, &u, &rho);
    keep[s] = (u < rho) ? 1u : 0u;
}

// Cell counters of the round's candidates: with few cells, millions of
// atomics on a handful of counters serialise in L2. Grids of at most
// kShCells cells count in shared memory per 1024-thread block and add one
// global atomic per touched cell.
constexpr uint32_t kShCells = 4096;
constexpr int kBinTPB = 1024;

// Compaction in stream order + cell counts.
__global__ void __launch_bounds__(kBinTPB) k_compact(const Real* __restrict__ reals, int R, const uint32_t* __restrict__ coff,
                          const uint64_t* __restrict__ kbeg, uint32_t nslots, const uint32_t* __restrict__ keep,
                          const uint32_t* __restrict__ kpos, float4* __restrict__ cpos, float4* __restrict__ cdir,
                          uint64_t* __restrict__ csidx, uint32_t* __restrict__ creal, uint32_t* __restrict__ ccell,
                          uint32_t* __restrict__ ccount, uint8_t* __restrict__ state, uint32_t ncell) {
    extern __shared__ uint32_t shc[];
    const bool bin = ccell != nullptr;  // the cell-stencil sweeps bin the candidates; the tube sweeps do not
    const bool sh = bin && ncell <= kShCells;
    if (sh) {
        for (uint32_t c = threadIdx.x; c < ncell; c += blockDim.x) shc[c] = 0;
        __syncthreads();
    }
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nslots && keep[s]) {
        int r = find_real(coff, R, s);
        const Real& Re = reals[r];
        uint64_t k = kbeg[r] + (s - coff[r]);
        float4 p, d;
        float u, rho;
        candidate(Re, k, &p, &d, &u, &rho);
        uint32_t c = kpos[s];
        cpos[c] = p;
        cdir[c] = d;
        csidx[c] = k;
        creal[c] = (uint32_t)r;
        state[c] = ST_ALIVE;
        if (bin) {
            const uint32_t cell = cell_of(Re, p.x, p.y, p.z);
            ccell[c] = cell;
            atomicAdd(sh ? &shc[cell] : &ccount[cell], 1u);
        }
    }
    if (sh) {
        __syncthreads();
        for (uint32_t c = threadIdx.x; c < ncell; c += blockDim.x)
            if (shc[c]) atomicAdd(&ccount[c], shc[c]);
    }
}

// Counting-sort scatter: perm[start[cell] + cursor] = id. With few cells the
// block ranks its ids per cell in shared memory and reserves one range per
// touched cell.
__global__ void __launch_bounds__(kBinTPB) k_bin(uint32_t n, const uint32_t* __restrict__ ntot, const uint32_t* __restrict__ cellof,
                      const uint32_t* __restrict__ start, uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm,
                      uint32_t ncell) {
    extern __shared__ uint32_t shb[];  // local count, then base, per cell
    const bool sh = ncell <= kShCells;
    if (sh) {
        for (uint32_t c = threadIdx.x; c < ncell; c += blockDim.x) shb[c] = 0;
        __syncthreads();
    }
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t m = ntot ? *ntot : n;
    const bool valid = i < m;
    uint32_t cell = 0, rank = 0;
    if (valid) {
        cell = cellof[i];
        rank = atomicAdd(sh ? &shb[cell] : &cursor[cell], 1u);
    }
    if (sh) {
        __syncthreads();
        for (uint32_t c = threadIdx.x; c < ncell; c += blockDim.x)
            shb[ncell + c] = shb[c] ? atomicAdd(&cursor[c], shb[c]) : 0u;
        __syncthreads();
        rank += shb[ncell + cell];
    }
    if (valid) perm[start[cell] + rank] = i;
}

// Candidate vs accepted rods of one neighbour cell (cuda_OldExtIsectLB's job),
// over the work list: each item is up to 32 candidates of a cell against up to
// kSeg rods of one neighbour cell. Each lane marks the staged rods that pass
// the capsule pre-test of its candidate; the marked pairs are evaluated by the
// whole warp: far pairs dropped, clear hits decided in FP32 (the candidate is
// rejected at once and skipped by every other item at its next tile), the
// rest queued for FP64 (probe = compact candidate id, target = sorted rod).
__global__ void __launch_bounds__(kTPB, 6) k_old_tiles(const Real* __restrict__ reals,
                                                    const uint32_t* __restrict__ nitems, uint32_t icap,
                                                    const Item* __restrict__ items,
                                                    const uint32_t* __restrict__ cperm,
                                                    const float4* __restrict__ gpos, const float4* __restrict__ gdir,
                                                    const float4* __restrict__ spos, const float4* __restrict__ sdir,
                                                    uint8_t* state, unsigned long long* __restrict__ xq,
                                                    unsigned long long xcap, unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ WarpTile tiles[kW];
    __shared__ float4 ppos[kW][32], pdir[kW][32];
    __shared__ uint32_t pcid[kW][32];
    __shared__ int msp[kW][32];
    __shared__ uint32_t msm[kW][32];
    __shared__ uint16_t mq2[kW][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpTile& T = tiles[w];
    volatile uint8_t* vst = state;
    unsigned long long tests = 0, cert = 0, nitem = 0, ntile = 0, nmark = 0, nline = 0;
    const uint32_t n = min(*nitems, icap);
    const uint32_t stride = gridDim.x * kW;
    Item nxt = blockIdx.x * kW + w < n ? items[blockIdx.x * kW + w] : Item{0, 0, 0, 0};
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += stride) {
        const Item I = nxt;
        if (it + stride < n) nxt = items[it + stride];  // next item's descriptor in flight meanwhile
        ++nitem;
        uint32_t np, nt;
        int img[3];
        item_unpack(I, &np, &nt, img);
        const Real& Re = reals[I.real];
        const bool have = (uint32_t)lane < np;
        const uint32_t q = I.pfirst + lane;
        const uint32_t cid = have ? cperm[q] : 0u;
        float4 pA = make_float4(0, 0, 0, 0), cA = pA;
        if (have) { pA = gpos[q]; cA = gdir[q]; }
        bool alive = have && vst[cid] != ST_REJ_OLD;
        __syncwarp();
        ppos[w][lane] = pA;
        pdir[w][lane] = cA;
        pcid[w][lane] = cid;
        const float sx = img[0] * Re.L[0], sy = img[1] * Re.L[1], sz = img[2] * Re.L[2];
        const float ax = pA.x - sx, ay = pA.y - sy, az = pA.z - sz;
        const float hA2 = (pA.w * 0.5f + cA.w + Re.eps + cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack;
        const float hAe = pA.w * 0.5f + cA.w + Re.eps;
        const float hC = (cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack + 4e-6f * (1.0f + hA2);
        // line bound of the marking loop: margin bounded with the pair's reach
        // (errA + 4e-6 hBt covers 4e-6 |b| + slack for any pair within reach),
        // threshold thA + a_B scf2, both sides squared
        const float errA = 4e-6f * (1.0f + hA2) + Re.slack;
        const float thA = (cA.w * Re.scf + Re.sep + Re.eps) * 1.0002f, scf2 = Re.scf * 1.0002f;
        unsigned dead = 0;  // probe lanes decided during this item (warp-uniform)
        for (uint32_t b = 0; b < nt; b += kWT) {
            if (!__any_sync(0xffffffffu, alive)) break;
            const uint32_t m = min((uint32_t)kWT, nt - b);
            if ((uint32_t)lane < m) {
                const uint32_t k = I.tfirst + b + lane;
                const float4 p = spos[k], c = sdir[k];
                T.l[lane] = p.w;
                T.p[lane] = make_float4(p.x, p.y, p.z, (p.w * 0.5f + c.w + Re.eps + c.w * Re.scf) * 1.000002f);
                T.c[lane] = c;
            } else {
                T.p[lane] = make_float4(kFar, kFar, kFar, 0.0f);
            }
            __syncwarp();
            uint32_t mask = 0;
            if (alive) {
                tests += m;
                const uint32_t m8 = (m + 7u) & ~7u;
                for (uint32_t j0 = 0; j0 < m8; j0 += 8) {
#pragma unroll
                    for (uint32_t jj = 0; jj < 8; ++jj) {
                        const float4 tq = T.p[j0 + jj];
                        const float bx = tq.x - ax, by = tq.y - ay, bz = tq.z - az;
                        // the axis lines certainly farther apart than the threshold (the
                        // test of line_far without its square root); near-parallel pairs
                        // are never far. Evaluated first: most staged pairs end here.
                        const float4 cB = T.c[j0 + jj];
                        const float nx = cA.y * cB.z - cA.z * cB.y;
                        const float ny = cA.z * cB.x - cA.x * cB.z;
                        const float nz = cA.x * cB.y - cA.y * cB.x;
                        const float nn = nx * nx + ny * ny + nz * nz;
                        const float nb = fabsf(nx * bx + ny * by + nz * bz) - fmaf(4e-6f, tq.w, errA);
                        const float thL = fmaf(cB.w, scf2, thA);
                        const bool lfar = nn > 1e-4f && nb > 0.0f && nb * nb > thL * thL * nn;
                        if (!lfar && capsule_near(bx, by, bz, cA.x, cA.y, cA.z, hAe, tq.w, hC)) mask |= 1u << (j0 + jj);
                    }
                }
            }
            const uint32_t base = I.tfirst + b;
            auto keep = [&](int pl, int t) {
                if ((dead >> pl) & 1u) return false;
                const float4 dA = pdir[w][pl], tq = T.p[t], cB = T.c[t];
                const float4 pB = make_float4(tq.x, tq.y, tq.z, T.l[t]);
                return !line_far(ppos[w][pl], dA, pB, cB, sx, sy, sz, (cB.w + dA.w) * Re.scf + Re.sep + Re.eps,
                                 Re.slack);
            };
            ++ntile;
            nmark += __popc(mask);
            const int kept_ = for_marked_pairs(mask, lane, msp[w], msm[w], mq2[w], keep, [&](bool valid, int pl, int t) {
                bool hit = false;
                if (valid && !((dead >> pl) & 1u)) {
                    const float4 qA = ppos[w][pl], dA = pdir[w][pl];
                    const float4 tq = T.p[t], cB = T.c[t];
                    const float4 pB = make_float4(tq.x, tq.y, tq.z, T.l[t]);
                    const float thr = (cB.w + dA.w) * Re.scf + Re.sep + Re.eps;
                    if (maybe_near(qA, dA, pB, cB, sx, sy, sz, thr, Re.eps, Re.slack)) {
                        const uint32_t c = pcid[w][pl];
                        if (!Re.typo && certain_hit(qA, dA, pB, cB, sx, sy, sz, thr, Re.eps, Re.slack)) {
                            hit = true;
                            ++cert;
                            vst[c] = ST_REJ_OLD;
                        } else {
                            xq_push(xq, xcap, &ctr[C_XQ_OLD], xq_pack(c, base + t, img));
                        }
                    }
                }
                dead |= __reduce_or_sync(0xffffffffu, hit ? (1u << pl) : 0u);
            });
            if (lane == 0) nline += kept_;
            if ((dead >> lane) & 1u) alive = false;
            if (alive && vst[cid] == ST_REJ_OLD) alive = false;  // decided by another item
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_PAIR_TESTS], tests);
    warp_add_u64(&ctr[C_CERT], cert);
    if (lane == 0) {
        atomicAdd(&ctr[C_G_ITEMS], nitem);
        atomicAdd(&ctr[C_G_TILES], ntile);
        atomicAdd(&ctr[C_G_LINE], nline);
    }
    warp_add_u64(&ctr[C_G_MARKED], nmark);
}

// FP64 decisions of the queued (candidate, accepted rod) pairs.
__global__ void __launch_bounds__(256) k_old_exact(const Real* __restrict__ reals,
                                                   const unsigned long long* __restrict__ xq,
                                                   const unsigned long long* __restrict__ first,
                                                   const unsigned long long* __restrict__ count,
                                                   unsigned long long cap, const float4* __restrict__ cpos,
                                                   const float4* __restrict__ cdir, const uint32_t* __restrict__ creal,
                                                   const float4* __restrict__ spos, const float4* __restrict__ sdir,
                                                   uint8_t* state, unsigned long long* __restrict__ ctr) {
    const unsigned long long n = min(*count, cap);
    const unsigned long long e0 = first ? min(*first, cap) : 0ull;
    volatile uint8_t* vst = state;
    unsigned long long exact = 0, flips = 0;
    for (unsigned long long e = e0 + blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t cid, j;
        int img[3];
        xq_unpack(xq[e], &cid, &j, img);
        if (vst[cid] == ST_REJ_OLD) continue;
        const Real& Re = reals[creal[cid]];
        const float4 pA = cpos[cid], cA = cdir[cid], pB = spos[j], cB = sdir[j];
        ++exact;
        const RodD a = rodd(pA, cA), b = rodd(pB, cB);
        double d = ref_distance_d(a, b, img[0] * (double)Re.L[0], img[1] * (double)Re.L[1],
                                  img[2] * (double)Re.L[2], (double)Re.eps, Re.typo != 0, nullptr, nullptr,
                                  nullptr, nullptr, nullptr);
        bool h = d < thresh_d(a.a, b.a, (double)Re.scf, (double)Re.sep, (double)Re.eps);
        const float thr = (cB.w + cA.w) * Re.scf + Re.sep + Re.eps;
        if (ref_hit_f32(pA, cA, pB, cB, img[0] * Re.L[0], img[1] * Re.L[1], img[2] * Re.L[2], Re.eps, thr,
                        Re.typo != 0) != h)
            ++flips;
        if (h) vst[cid] = ST_REJ_OLD;
    }
    warp_add_u64(&ctr[C_EXACT], exact);
    warp_add_u64(&ctr[C_FLIPS], flips);
}

// Survivors of the old-rod test, binned by cell (stream order is kept in the
// per-candidate key): the in-round conflict sweep runs over these only.
// Warp-aggregated increment of ctr[key] for the active lanes (lanes of a
// warp that share a key add once); returns each lane's slot. Every lane of
// the warp calls it.
__device__ __forceinline__ uint32_t warp_agg_inc(uint32_t* ctr, uint32_t key, bool active) {
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if (!active) return 0u;
    const unsigned peers = __match_any_sync(act, key);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    uint32_t base = 0u;
    if (lane == leader) base = atomicAdd(&ctr[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

// Survivors per cell; the walk is in cell order, so a warp's lanes mostly
// share one counter and add to it once.
__global__ void k_alive_count(uint32_t n, const uint32_t* __restrict__ ntot, const uint32_t* __restrict__ cperm,
                              const uint8_t* __restrict__ state, const uint32_t* __restrict__ ccell,
                              uint32_t* __restrict__ acount) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    bool alive = false;
    uint32_t cell = 0;
    if (q < *ntot) {
        const uint32_t cid = cperm[q];
        alive = state[cid] == ST_ALIVE;
        cell = ccell[cid];
    }
    (void)warp_agg_inc(acount, cell, alive);
}
__global__ void k_alive_bin(uint32_t n, const uint32_t* __restrict__ ntot, const uint32_t* __restrict__ cperm,
                            const uint8_t* __restrict__ state, const uint32_t* __restrict__ ccell,
                            const uint32_t* __restrict__ astart, uint32_t* __restrict__ acur,
                            const float4* __restrict__ gpos, const float4* __restrict__ gdir,
                            uint32_t* __restrict__ aperm, float4* __restrict__ apos,
                            float4* __restrict__ adir) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    bool alive = false;
    uint32_t cid = 0, cell = 0;
    if (q < *ntot) {
        cid = cperm[q];
        alive = state[cid] == ST_ALIVE;
        cell = ccell[cid];
    }
    const uint32_t slot = warp_agg_inc(acur, cell, alive);
    if (!alive) return;
    const uint32_t d = astart[cell] + slot;
    aperm[d] = cid;
    apos[d] = gpos[q];
    adir[d] = gdir[q];
}

// Earlier survivors of one neighbour cell that a survivor hits, over the work
// list of the survivor cells (capsule marks per lane, full-warp evaluation of
// the marked pairs). Compact candidate ids follow stream order within a
// realisation, so "earlier" is a smaller id. Certified hits are listed
// directly, uncertain pairs queued (target = compact candidate id).
__global__ void __launch_bounds__(kTPB, 6) k_conf_tiles(const Real* __restrict__ reals,
                                                     const uint32_t* __restrict__ nitems, uint32_t icap,
                                                     const Item* __restrict__ items,
                                                     const uint32_t* __restrict__ aperm,
                                                     const float4* __restrict__ apos, const float4* __restrict__ adir,
                                                     uint32_t* __restrict__ ccnt, uint32_t* __restrict__ clist,
                                                     unsigned long long* __restrict__ xq, unsigned long long xcap,
                                                     unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ WarpTile tiles[kW];
    __shared__ uint32_t tid_[kW][kWT];
    __shared__ float4 ppos[kW][32], pdir[kW][32];
    __shared__ uint32_t pcid[kW][32];
    __shared__ int msp[kW][32];
    __shared__ uint32_t msm[kW][32];
    __shared__ uint16_t mq2[kW][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpTile& T = tiles[w];
    unsigned long long tests = 0, ovf = 0, cert = 0, nitem = 0, ntile = 0, nmark = 0, nline = 0;
    const uint32_t n = min(*nitems, icap);
    const uint32_t stride = gridDim.x * kW;
    Item nxt = blockIdx.x * kW + w < n ? items[blockIdx.x * kW + w] : Item{0, 0, 0, 0};
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += stride) {
        const Item I = nxt;
        if (it + stride < n) nxt = items[it + stride];  // next item's descriptor in flight meanwhile
        ++nitem;
        uint32_t np, nt;
        int img[3];
        item_unpack(I, &np, &nt, img);
        const Real& Re = reals[I.real];
        const bool have = (uint32_t)lane < np;
        const uint32_t q = I.pfirst + lane;
        const uint32_t cid = have ? aperm[q] : 0u;
        float4 pA = make_float4(0, 0, 0, 0), cA = pA;
        if (have) { pA = apos[q]; cA = adir[q]; }
        __syncwarp();
        ppos[w][lane] = pA;
        pdir[w][lane] = cA;
        pcid[w][lane] = cid;
        const float sx = img[0] * Re.L[0], sy = img[1] * Re.L[1], sz = img[2] * Re.L[2];
        const float ax = pA.x - sx, ay = pA.y - sy, az = pA.z - sz;
        const float hA2 = (pA.w * 0.5f + cA.w + Re.eps + cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack;
        const float hAe = pA.w * 0.5f + cA.w + Re.eps;
        const float hC = (cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack + 4e-6f * (1.0f + hA2);
        for (uint32_t b = 0; b < nt; b += kWT) {
            const uint32_t m = min((uint32_t)kWT, nt - b);
            if ((uint32_t)lane < m) {
                const uint32_t k = I.tfirst + b + lane;
                const float4 p = apos[k], c = adir[k];
                T.l[lane] = p.w;
                T.p[lane] = make_float4(p.x, p.y, p.z, (p.w * 0.5f + c.w + Re.eps + c.w * Re.scf) * 1.000002f);
                T.c[lane] = c;
                tid_[w][lane] = aperm[k];
            } else {
                T.p[lane] = make_float4(kFar, kFar, kFar, 0.0f);
                tid_[w][lane] = 0xffffffffu;
            }
            __syncwarp();
            uint32_t mask = 0, emask = 0;  // marked pairs; earlier survivors
            if (have) {
                const uint32_t m8 = (m + 7u) & ~7u;
                for (uint32_t j0 = 0; j0 < m8; j0 += 8) {
#pragma unroll
                    for (uint32_t jj = 0; jj < 8; ++jj) {
                        const uint32_t j = j0 + jj;
                        const float4 tq = T.p[j];
                        const float bx = tq.x - ax, by = tq.y - ay, bz = tq.z - az;
                        const uint32_t bit = tid_[w][j] < cid ? (1u << j) : 0u;
                        emask |= bit;
                        if (capsule_near(bx, by, bz, cA.x, cA.y, cA.z, hAe, tq.w, hC)) mask |= bit;
                    }
                }
                tests += __popc(emask);
            }
            auto keep = [&](int pl, int t) {
                const float4 dA = pdir[w][pl], tq = T.p[t], cB = T.c[t];
                const float4 pB = make_float4(tq.x, tq.y, tq.z, T.l[t]);
                return !line_far(ppos[w][pl], dA, pB, cB, sx, sy, sz, (cB.w + dA.w) * Re.scf + Re.sep + Re.eps,
                                 Re.slack);
            };
            ++ntile;
            nmark += __popc(mask);
            const int kept_ = for_marked_pairs(mask, lane, msp[w], msm[w], mq2[w], keep, [&](bool valid, int pl, int t) {
                if (!valid) return;
                const float4 qA = ppos[w][pl], dA = pdir[w][pl];
                const float4 tq = T.p[t], cB = T.c[t];
                const float4 pB = make_float4(tq.x, tq.y, tq.z, T.l[t]);
                const float thr = (cB.w + dA.w) * Re.scf + Re.sep + Re.eps;
                if (maybe_near(qA, dA, pB, cB, sx, sy, sz, thr, Re.eps, Re.slack)) {
                    const uint32_t c = pcid[w][pl];
                    if (!Re.typo && certain_hit(qA, dA, pB, cB, sx, sy, sz, thr, Re.eps, Re.slack)) {
                        ++cert;
                        uint32_t slot = atomicAdd(&ccnt[c], 1u);
                        if (slot < (uint32_t)kConflictCap) clist[(size_t)c * kConflictCap + slot] = tid_[w][t];
                        else ++ovf;
                    } else {
                        xq_push(xq, xcap, &ctr[C_XQ_CONF], xq_pack(c, tid_[w][t], img));
                    }
                }
            });
            if (lane == 0) nline += kept_;
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_PAIR_TESTS], tests);
    warp_add_u64(&ctr[C_OVERFLOW], ovf);
    warp_add_u64(&ctr[C_CERT], cert);
    if (lane == 0) {
        atomicAdd(&ctr[C_G_ITEMS], nitem);
        atomicAdd(&ctr[C_G_TILES], ntile);
        atomicAdd(&ctr[C_G_LINE], nline);
    }
    warp_add_u64(&ctr[C_G_MARKED], nmark);
}

__global__ void __launch_bounds__(256) k_conf_exact(const Real* __restrict__ reals,
                                                    const unsigned long long* __restrict__ xq,
                                                    const uint32_t* __restrict__ xqc,
                                                    const unsigned long long* __restrict__ count,
                                                    unsigned long long cap, const float4* __restrict__ cpos,
                                                    const float4* __restrict__ cdir, const uint32_t* __restrict__ creal,
                                                    uint32_t* __restrict__ ccnt, uint32_t* __restrict__ clist,
                                                    unsigned long long* __restrict__ ctr) {
    const unsigned long long n = min(*count, cap);
    unsigned long long exact = 0, flips = 0, ovf = 0;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t cid, j;
        int img[3];
        xq_unpack(xq[e], &cid, &j, img);
        const Real& Re = reals[creal[cid]];
        const float4 pA = cpos[cid], cA = cdir[cid], pB = cpos[j], cB = cdir[j];
        ++exact;
        const RodD a = rodd(pA, cA), b = rodd(pB, cB);
        const double sx = img[0] * (double)Re.L[0], sy = img[1] * (double)Re.L[1], sz = img[2] * (double)Re.L[2];
        double t0d, t1d;
        double d = ref_distance_d(a, b, sx, sy, sz, (double)Re.eps, Re.typo != 0, &t0d, &t1d, nullptr, nullptr,
                                  nullptr);
        bool h = d < thresh_d(a.a, b.a, (double)Re.scf, (double)Re.sep, (double)Re.eps);
        // tube sweeps: a pair queued from several cells is listed by the one
        // holding the midpoint of its points
        if (xqc && h && !tube_claims_d(Re, Re.per_gen, xqc[e], a, b, sx, sy, sz, t0d, t1d)) continue;
        const float thr = (cB.w + cA.w) * Re.scf + Re.sep + Re.eps;
        if (ref_hit_f32(pA, cA, pB, cB, img[0] * Re.L[0], img[1] * Re.L[1], img[2] * Re.L[2], Re.eps, thr,
                        Re.typo != 0) != h)
            ++flips;
        if (h) {
            uint32_t slot = atomicAdd(&ccnt[cid], 1u);
            if (slot < (uint32_t)kConflictCap) clist[(size_t)cid * kConflictCap + slot] = j;
            else ++ovf;
        }
    }
    warp_add_u64(&ctr[C_EXACT], exact);
    warp_add_u64(&ctr[C_FLIPS], flips);
    warp_add_u64(&ctr[C_OVERFLOW], ovf);
}

// ---------------------------------------------------------------------------
// Tube sweeps of the generation (nf_tube.cuh): the pairs registered together
// in a tube cell. A cell item is (<= 32 probe entries, <= kTSeg target
// entries) of one cell: a lane holds a probe, the warp stages 32 targets at a
// time. A packed item holds the small cells of a run of consecutive cells
// (<= 32 probes and <= 32 targets in all): a lane holds a probe of any of
// them and tests it against its own cell's targets (a range of the one
// staged tile). Every entry carries the image of its object's copy in the
// cell: the marking loop works on the copies, the filters and the FP64 queue
// on the original coordinates with the relative image (target copy image -
// probe copy image). An item's cells belong to one realisation (carried in
// the item); per-pair cells come from the probe lane. The marking test is the
// line bound and then the capsule test (pair-parallel), so the hand-out's
// first stage only drops pairs whose relative image is out of range; the
// full filter, certificate and FP64 queue follow as in the stencil kernels.
// The rods' cells are [start, start + count) (the registration leaves room
// for the rods of later rounds).
// ---------------------------------------------------------------------------

// Candidates (probe entries) against placed rods (target entries) of one tube
// cell: cuda_OldExtIsectLB's job (inc/intersection_kern.h:245-364) on the
// tube grid.
__global__ void __launch_bounds__(kTPB, 8) k_tube_old(const Real* __restrict__ reals, int R,
                                                   const uint32_t* __restrict__ toffs,
                                                   const uint32_t* __restrict__ nitems, uint32_t icap,
                                                   const TItem* __restrict__ items,
                                                   const uint32_t* __restrict__ pstart,
                                                   const uint32_t* __restrict__ tstart,
                                                   const uint32_t* __restrict__ tcnt,
                                                   const uint32_t* __restrict__ pent,
                                                   const float4* __restrict__ cpos, const float4* __restrict__ cdir,
                                                   const uint32_t* __restrict__ tent,
                                                   const float4* __restrict__ rpos, const float4* __restrict__ rdir,
                                                   uint8_t* state, unsigned long long* __restrict__ xq,
                                                   unsigned long long xcap, unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ TubeTile tiles[kW];
    __shared__ TubePack packs[kW];
    __shared__ float4 ppos[kW][32], pdir[kW][32];
    __shared__ uint32_t pcid[kW][32], pim[kW][32];
    __shared__ int msp[kW][32];
    __shared__ uint32_t msm[kW][32];
    __shared__ uint16_t mq2[kW][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    TubeTile& T = tiles[w];
    volatile uint8_t* vst = state;
    unsigned long long tests = 0, cert = 0, nitem = 0, ntile = 0, nmark = 0, nline = 0;
    const uint32_t n = min(*nitems, icap);
    const uint32_t stride = gridDim.x * kW;
    TItem nxt = blockIdx.x * kW + w < n ? items[blockIdx.x * kW + w] : TItem{0, 0, 0, 0};
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += stride) {
        const TItem I = nxt;
        if (it + stride < n) nxt = items[it + stride];
        ++nitem;
        const TubeLane L = tube_lane(I, lane, pstart, tstart, nullptr, tcnt, packs[w]);
        const int rl = item_real(I.pfirst, I.cnt, I.cell, toffs, R);
        const Real& Re = reals[rl];
        const bool have = (uint32_t)lane < L.np;
        uint32_t cid = 0, ipc = 0;
        float4 pA = make_float4(0, 0, 0, 0), cA = pA;
        if (have) {
            const uint32_t e = pent[L.pe];
            cid = e >> kTubeIdShift;
            ipc = e & 63u;
            pA = cpos[L.pe];
            cA = cdir[L.pe];
        }
        bool alive = have && vst[cid] != ST_REJ_OLD;
        __syncwarp();
        ppos[w][lane] = pA;
        pdir[w][lane] = cA;
        pcid[w][lane] = cid;
        pim[w][lane] = ipc;
        int ia[3];
        img_of(ipc, ia);
        // the probe's copy in this cell
        const float ax = pA.x + ia[0] * Re.L[0], ay = pA.y + ia[1] * Re.L[1], az = pA.z + ia[2] * Re.L[2];
        const float hA2 = (pA.w * 0.5f + cA.w + Re.eps + cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack;
        const float hAe = pA.w * 0.5f + cA.w + Re.eps;
        const float hC = (cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack + 4e-6f * (1.0f + hA2);
        const float errA = 4e-6f * (1.0f + hA2) + 2.0f * Re.slack;
        const float thA = (cA.w * Re.scf + Re.sep + Re.eps) * 1.0002f, scf2 = Re.scf * 1.0002f;
        unsigned dead = 0;
        for (uint32_t b = 0; b < L.nt; b += kWT) {
            if (!__any_sync(0xffffffffu, alive)) break;
            const uint32_t m = min((uint32_t)kWT, L.nt - b);
            if ((uint32_t)lane < m) {
                uint32_t tc;
                const uint32_t q = tube_target(I, L, packs[w], b, (uint32_t)lane, &tc);
                const Real& Rt = Re;  // an item's cells belong to one realisation
                (void)tc;
                const uint32_t e = tent[q];
                const uint32_t k = e >> kTubeIdShift;
                const float4 p = rpos[q], c = rdir[q];
                int ib[3];
                img_of(e & 63u, ib);
                T.p[lane] = p;
                T.ps[lane] = make_float4(p.x + ib[0] * Rt.L[0], p.y + ib[1] * Rt.L[1], p.z + ib[2] * Rt.L[2],
                                         (p.w * 0.5f + c.w + Rt.eps + c.w * Rt.scf) * 1.000002f);
                T.c[lane] = c;
                T.id[lane] = k;
                T.im[lane] = e & 63u;
            } else {
                T.ps[lane] = make_float4(kFar, kFar, kFar, 0.0f);
            }
            __syncwarp();
            if (b == 0 && it + stride < n) {  // the next item's first loads, into L2
                const uint32_t span = nxt.cnt & 63u;
                if ((uint32_t)lane < span) {
                    if (!(nxt.cnt & kPackBit)) {
                        const uint32_t q = nxt.pfirst + (uint32_t)lane;
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(pent + q));
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(cpos + q));
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(cdir + q));
                    } else {
                        const uint32_t c = nxt.cell + (uint32_t)lane;
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(pstart + c));
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(tstart + c));
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(tcnt + c));
                    }
                }
            }
            const uint32_t lo = L.packed ? L.tlo : 0u, len = L.packed ? L.tlen : m;
            if (alive) tests += len;
            // Pair-parallel marking: the na live probes take 2^s >= na lanes
            // each (slot = lane mod 2^s); a lane tests its slot's probe
            // against every (32 >> s)-th target of the probe's range, and the
            // lanes of a slot OR their marks together for the probe's lane.
            const unsigned am = __ballot_sync(0xffffffffu, alive);
            const int na = __popc(am);
            const int sh = na <= 1 ? 0 : 32 - __clz(na - 1);
            const int slot = lane & ((1 << sh) - 1);
            const bool qv = slot < na;
            const int src = qv ? nth_set_bit(am, slot) : lane;
            const float qx = __shfl_sync(0xffffffffu, ax, src), qy = __shfl_sync(0xffffffffu, ay, src),
                        qz = __shfl_sync(0xffffffffu, az, src);
            const float qcx = __shfl_sync(0xffffffffu, cA.x, src), qcy = __shfl_sync(0xffffffffu, cA.y, src),
                        qcz = __shfl_sync(0xffffffffu, cA.z, src);
            const float qh = __shfl_sync(0xffffffffu, hAe, src), qC = __shfl_sync(0xffffffffu, hC, src);
            const float qerr = __shfl_sync(0xffffffffu, errA, src), qth = __shfl_sync(0xffffffffu, thA, src);
            const uint32_t qlo = __shfl_sync(0xffffffffu, lo, src);
            const uint32_t qlen0 = __shfl_sync(0xffffffffu, len, src);
            const uint32_t qlen = qv ? qlen0 : 0u;
            const uint32_t step = 32u >> sh;
            uint32_t qmask = 0;
            for (uint32_t u0 = (uint32_t)lane >> sh; u0 < qlen; u0 += 4u * step) {
#pragma unroll
                for (uint32_t jj = 0; jj < 4; ++jj) {
                    const uint32_t u = u0 + jj * step;
                    if (u < qlen) {
                        const uint32_t j = qlo + u;
                        const float4 tq = T.ps[j];
                        const float bx = tq.x - qx, by = tq.y - qy, bz = tq.z - qz;
                        const float4 cB = T.c[j];
                        const float nx = qcy * cB.z - qcz * cB.y;
                        const float ny = qcz * cB.x - qcx * cB.z;
                        const float nz = qcx * cB.y - qcy * cB.x;
                        const float nn = nx * nx + ny * ny + nz * nz;
                        const float nb = fabsf(nx * bx + ny * by + nz * bz) - fmaf(4e-6f, tq.w, qerr);
                        const float thL = fmaf(cB.w, scf2, qth);
                        const bool lfar = nn > 1e-4f && nb > 0.0f && nb * nb > thL * thL * nn;
                        if (!lfar && capsule_near(bx, by, bz, qcx, qcy, qcz, qh, tq.w, qC)) qmask |= 1u << j;
                    }
                }
            }
            for (int o = 1 << sh; o < 32; o <<= 1) qmask |= __shfl_xor_sync(0xffffffffu, qmask, o);
            const uint32_t mine = __shfl_sync(0xffffffffu, qmask, __popc(am & ((1u << lane) - 1u)));
            const uint32_t mask = alive ? mine : 0u;
            auto keep = [&](int pl, int t) {
                if ((dead >> pl) & 1u) return false;
                int img[3];
                return rel_img(pim[w][pl], T.im[t], img);
            };
            ++ntile;
            nmark += __popc(mask);
            const int kept_ = for_marked_pairs(mask, lane, msp[w], msm[w], mq2[w], keep, [&](bool valid, int pl, int t) {
                bool hit = false;
                if (valid && !((dead >> pl) & 1u)) {
                    const Real& Rp = Re;
                    const float4 qA = ppos[w][pl], dA = pdir[w][pl];
                    const float4 pB = T.p[t], cB = T.c[t];
                    int img[3];
                    rel_img(pim[w][pl], T.im[t], img);
                    const float sx = img[0] * Rp.L[0], sy = img[1] * Rp.L[1], sz = img[2] * Rp.L[2];
                    const float thr = (cB.w + dA.w) * Rp.scf + Rp.sep + Rp.eps;
                    if (maybe_near(qA, dA, pB, cB, sx, sy, sz, thr, Rp.eps, Rp.slack)) {
                        const uint32_t c = pcid[w][pl];
                        if (!Rp.typo && certain_hit(qA, dA, pB, cB, sx, sy, sz, thr, Rp.eps, Rp.slack)) {
                            hit = true;
                            ++cert;
                            vst[c] = ST_REJ_OLD;
                        } else {
                            xq_push(xq, xcap, &ctr[C_XQ_OLD], xq_pack(c, T.id[t], img));
                        }
                    }
                }
                dead |= __reduce_or_sync(0xffffffffu, hit ? (1u << pl) : 0u);
            });
            if (lane == 0) nline += kept_;
            if ((dead >> lane) & 1u) alive = false;
            if (alive && vst[cid] == ST_REJ_OLD) alive = false;
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_PAIR_TESTS], tests);
    warp_add_u64(&ctr[C_CERT], cert);
    if (lane == 0) {
        atomicAdd(&ctr[C_G_ITEMS], nitem);
        atomicAdd(&ctr[C_G_TILES], ntile);
        atomicAdd(&ctr[C_G_LINE], nline);
    }
    warp_add_u64(&ctr[C_G_MARKED], nmark);
}

// Survivors against earlier survivors of one tube cell (probe and target
// entries are the same list, so every pair is tested once, in whichever
// order it is met, and evaluated with the later survivor as the probe):
// k_conf_tiles on the tube grid. A certified hit
// is listed by the one cell that claims it (tube_claims), so no pair enters a
// conflict list twice from the FP32 path; uncertain pairs are queued from
// every cell they share (the FP64 pass may list a pair again, which the
// resolution ignores).
__global__ void __launch_bounds__(kTPB, 7) k_tube_conf(const Real* __restrict__ reals, int R,
                                                    const uint32_t* __restrict__ toffs,
                                                    const uint32_t* __restrict__ nitems, uint32_t icap,
                                                    const TItem* __restrict__ items,
                                                    const uint32_t* __restrict__ start,
                                                    const uint32_t* __restrict__ cnt,
                                                    const uint32_t* __restrict__ ent,
                                                    const float4* __restrict__ cpos, const float4* __restrict__ cdir,
                                                    uint32_t* __restrict__ ccnt, uint32_t* __restrict__ clist,
                                                    unsigned long long* __restrict__ xq, uint32_t* __restrict__ xqc,
                                                    unsigned long long xcap, unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ TubeTile tiles[kW];
    __shared__ TubePack packs[kW];
    __shared__ float4 ppos[kW][32], pdir[kW][32];
    __shared__ uint32_t pcid[kW][32], pim[kW][32], pcel[kW][32];
    __shared__ int msp[kW][32];
    __shared__ uint32_t msm[kW][32];
    __shared__ uint16_t mq2[kW][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    TubeTile& T = tiles[w];
    unsigned long long tests = 0, ovf = 0, cert = 0, nitem = 0, ntile = 0, nmark = 0, nline = 0;
    const uint32_t n = min(*nitems, icap);
    const uint32_t stride = gridDim.x * kW;
    TItem nxt = blockIdx.x * kW + w < n ? items[blockIdx.x * kW + w] : TItem{0, 0, 0, 0};
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += stride) {
        const TItem I = nxt;
        if (it + stride < n) nxt = items[it + stride];
        ++nitem;
        const TubeLane L = tube_lane(I, lane, start, start, cnt, cnt, packs[w]);
        const int rl = item_real(I.pfirst, I.cnt, I.cell, toffs, R);
        const Real& Re = reals[rl];
        const bool have = (uint32_t)lane < L.np;
        uint32_t cid = 0, ipc = 0;
        float4 pA = make_float4(0, 0, 0, 0), cA = pA;
        if (have) {
            const uint32_t e = ent[L.pe];
            cid = e >> kTubeIdShift;
            ipc = e & 63u;
            pA = cpos[L.pe];
            cA = cdir[L.pe];
        }
        __syncwarp();
        ppos[w][lane] = pA;
        pdir[w][lane] = cA;
        pcid[w][lane] = cid;
        pim[w][lane] = ipc;
        pcel[w][lane] = L.cell;
        int ia[3];
        img_of(ipc, ia);
        const float ax = pA.x + ia[0] * Re.L[0], ay = pA.y + ia[1] * Re.L[1], az = pA.z + ia[2] * Re.L[2];
        const float hA2 = (pA.w * 0.5f + cA.w + Re.eps + cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + Re.slack;
        const float hAe = pA.w * 0.5f + cA.w + Re.eps;
        const float hC = (cA.w * Re.scf + Re.sep + Re.eps) * 1.000002f + 2.0f * Re.slack + 4e-6f * (1.0f + hA2);
        const float errA = 4e-6f * (1.0f + hA2) + 2.0f * Re.slack;
        const float thA = (cA.w * Re.scf + Re.sep + Re.eps) * 1.0002f, scf2 = Re.scf * 1.0002f;
        for (uint32_t b = 0; b < L.nt; b += kWT) {
            const uint32_t m = min((uint32_t)kWT, L.nt - b);
            // Each pair once: probe and target entries are one list, so a
            // cell item's tiles before its probe chunk are left to the items
            // whose chunk they are; on the chunk's own tile (and in packed
            // items, where probe lane p is target slot p) a probe tests the
            // next half of its range, cyclically; tiles after the chunk are
            // tested whole. The evaluation takes the later survivor as the
            // probe of the pair.
            if (!L.packed && I.tfirst + b < I.pfirst) continue;
            const bool self = L.packed || I.tfirst + b == I.pfirst;
            if ((uint32_t)lane < m) {
                uint32_t tc;
                const uint32_t q = tube_target(I, L, packs[w], b, (uint32_t)lane, &tc);
                const Real& Rt = Re;  // an item's cells belong to one realisation
                (void)tc;
                const uint32_t e = ent[q];
                const uint32_t k = e >> kTubeIdShift;
                const float4 p = cpos[q], c = cdir[q];
                int ib[3];
                img_of(e & 63u, ib);
                T.p[lane] = p;
                T.ps[lane] = make_float4(p.x + ib[0] * Rt.L[0], p.y + ib[1] * Rt.L[1], p.z + ib[2] * Rt.L[2],
                                         (p.w * 0.5f + c.w + Rt.eps + c.w * Rt.scf) * 1.000002f);
                T.c[lane] = c;
                T.id[lane] = k;
                T.im[lane] = e & 63u;
            } else {
                T.ps[lane] = make_float4(kFar, kFar, kFar, 0.0f);
                T.id[lane] = 0xffffffffu;
            }
            __syncwarp();
            const uint32_t lo = L.packed ? L.tlo : 0u, len = L.packed ? L.tlen : m;
            // pair-parallel marking as in k_tube_old (every probe of the item)
            const int na = (int)L.np;
            const int sh = na <= 1 ? 0 : 32 - __clz(na - 1);
            const int slot = lane & ((1 << sh) - 1);
            const bool qv = slot < na;
            const int src = qv ? slot : lane;
            const float qx = __shfl_sync(0xffffffffu, ax, src), qy = __shfl_sync(0xffffffffu, ay, src),
                        qz = __shfl_sync(0xffffffffu, az, src);
            const float qcx = __shfl_sync(0xffffffffu, cA.x, src), qcy = __shfl_sync(0xffffffffu, cA.y, src),
                        qcz = __shfl_sync(0xffffffffu, cA.z, src);
            const float qh = __shfl_sync(0xffffffffu, hAe, src), qC = __shfl_sync(0xffffffffu, hC, src);
            const float qerr = __shfl_sync(0xffffffffu, errA, src), qth = __shfl_sync(0xffffffffu, thA, src);
            const uint32_t qcid = __shfl_sync(0xffffffffu, cid, src);
            const uint32_t qlo = __shfl_sync(0xffffffffu, lo, src);
            const uint32_t qlen0 = __shfl_sync(0xffffffffu, len, src);
            const uint32_t qlen = qv ? qlen0 : 0u;
            const uint32_t step = 32u >> sh;
            // on a self tile the probe (slot = its target slot) tests the
            // half of its range that follows it: nd targets from xl + 1 on
            const uint32_t xl = (uint32_t)src - qlo;
            const uint32_t nd = !self ? qlen : (qlen ? (qlen - 1u) / 2u + ((qlen & 1u) == 0u && xl < qlen / 2u) : 0u);
            uint32_t qmask = 0;  // marked pairs
            for (uint32_t u0 = (uint32_t)lane >> sh; u0 < nd; u0 += 4u * step) {
#pragma unroll
                for (uint32_t jj = 0; jj < 4; ++jj) {
                    const uint32_t u = u0 + jj * step;
                    if (u < nd) {
                        uint32_t y = self ? xl + 1u + u : u;
                        if (y >= qlen) y -= qlen;
                        const uint32_t j = qlo + y;
                        ++tests;
                        const float4 tq = T.ps[j];
                        const float bx = tq.x - qx, by = tq.y - qy, bz = tq.z - qz;
                        const uint32_t bit = 1u << j;
                        const float4 cB = T.c[j];
                        const float nx = qcy * cB.z - qcz * cB.y;
                        const float ny = qcz * cB.x - qcx * cB.z;
                        const float nz = qcx * cB.y - qcy * cB.x;
                        const float nn = nx * nx + ny * ny + nz * nz;
                        const float nb = fabsf(nx * bx + ny * by + nz * bz) - fmaf(4e-6f, tq.w, qerr);
                        const float thL = fmaf(cB.w, scf2, qth);
                        const bool lfar = nn > 1e-4f && nb > 0.0f && nb * nb > thL * thL * nn;
                        if (!lfar && capsule_near(bx, by, bz, qcx, qcy, qcz, qh, tq.w, qC)) qmask |= bit;
                    }
                }
            }
            for (int o = 1 << sh; o < 32; o <<= 1) qmask |= __shfl_xor_sync(0xffffffffu, qmask, o);
            const uint32_t mask = have ? qmask : 0u;
            auto keep = [&](int pl, int t) {
                int img[3];
                return rel_img(pim[w][pl], T.im[t], img);
            };
            ++ntile;
            nmark += __popc(mask);
            const int kept_ = for_marked_pairs(mask, lane, msp[w], msm[w], mq2[w], keep, [&](bool valid, int pl, int t) {
                if (!valid) return;
                const Real& Rp = Re;
                // the later survivor is the pair's probe (it lists the pair)
                const bool sw = T.id[t] > pcid[w][pl];
                const float4 qA = sw ? T.p[t] : ppos[w][pl], dA = sw ? T.c[t] : pdir[w][pl];
                const float4 pB = sw ? ppos[w][pl] : T.p[t], cB = sw ? pdir[w][pl] : T.c[t];
                int img[3];
                rel_img(pim[w][pl], T.im[t], img);
                if (sw) {
                    img[0] = -img[0];
                    img[1] = -img[1];
                    img[2] = -img[2];
                }
                const float sx = img[0] * Rp.L[0], sy = img[1] * Rp.L[1], sz = img[2] * Rp.L[2];
                const float thr = (cB.w + dA.w) * Rp.scf + Rp.sep + Rp.eps;
                if (maybe_near(qA, dA, pB, cB, sx, sy, sz, thr, Rp.eps, Rp.slack)) {
                    const uint32_t c = sw ? T.id[t] : pcid[w][pl], other = sw ? pcid[w][pl] : T.id[t];
                    const uint32_t cell = pcel[w][pl];
                    float t0 = 0.0f, t1 = 0.0f;
                    if (!Rp.typo && certain_hit(qA, dA, pB, cB, sx, sy, sz, thr, Rp.eps, Rp.slack, &t0, &t1)) {
                        // listed once: by the cell of the midpoint of the two feet
                        if (tube_claims(Rp, Rp.per_gen, cell, sw ? T.im[t] : pim[w][pl], qA, dA, pB, cB, sx, sy, sz,
                                        t0, t1)) {
                            ++cert;
                            uint32_t slot = atomicAdd(&ccnt[c], 1u);
                            if (slot < (uint32_t)kConflictCap) clist[(size_t)c * kConflictCap + slot] = other;
                            else ++ovf;
                        }
                    } else {
                        xq_push_cell(xq, xqc, xcap, &ctr[C_XQ_CONF], xq_pack(c, other, img), cell);
                    }
                }
            });
            if (lane == 0) nline += kept_;
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_PAIR_TESTS], tests);
    warp_add_u64(&ctr[C_OVERFLOW], ovf);
    warp_add_u64(&ctr[C_CERT], cert);
    if (lane == 0) {
        atomicAdd(&ctr[C_G_ITEMS], nitem);
        atomicAdd(&ctr[C_G_TILES], ntile);
        atomicAdd(&ctr[C_G_LINE], nline);
    }
    warp_add_u64(&ctr[C_G_MARKED], nmark);
}

// In-order resolution: a surviving candidate is rejected once one of its
// earlier conflicts is accepted and accepted once all of them are rejected.
// States only move from ST_ALIVE to a final state, so the passes need no grid
// barrier: a thread re-reads its conflicts up to `passes` times (with a short
// pause for the other threads to decide), and a candidate still open after
// that is counted in C_UNDECIDED (a count that is too high only costs the
// host another launch).
__global__ void k_resolve(const uint32_t* __restrict__ ntot, uint8_t* state, const uint32_t* __restrict__ ccnt,
                          const uint32_t* __restrict__ clist, unsigned long long* __restrict__ ctr, int passes) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= *ntot) return;
    volatile uint8_t* vs = state;
    if (vs[c] != ST_ALIVE) return;
    const uint32_t n = min(ccnt[c], (uint32_t)kConflictCap);
    for (int p = 0; p < passes; ++p) {
        bool any_acc = false, all_rej = true;
        for (uint32_t e = 0; e < n; ++e) {
            uint8_t s = vs[clist[(size_t)c * kConflictCap + e]];
            if (s == ST_ACC) { any_acc = true; break; }
            if (s == ST_ALIVE) all_rej = false;
        }
        if (any_acc) { vs[c] = ST_REJ_CONF; return; }
        if (all_rej) { vs[c] = ST_ACC; return; }
        __nanosleep(200);
    }
    atomicAdd(&ctr[C_UNDECIDED], 1ull);
}

__global__ void k_accflag(const uint32_t* __restrict__ ntot, uint32_t cap, const uint8_t* __restrict__ state,
                          uint32_t* __restrict__ accf) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cap) return;
    accf[c] = (c < *ntot && state[c] == ST_ACC) ? 1u : 0u;
}

// Per-realisation metadata of the round: meta[r*4 + {0:cfirst, 1:clast, 2:accbase, 3:acctot}].
__global__ void k_meta(int R, const uint32_t* __restrict__ coff, const uint32_t* __restrict__ keep,
                       const uint32_t* __restrict__ kpos, const uint32_t* __restrict__ accf,
                       const uint32_t* __restrict__ accpos, uint32_t* __restrict__ meta) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    uint32_t s0 = coff[r], s1 = coff[r + 1];
    uint32_t c0 = kpos[s0];
    uint32_t c1 = (s1 > s0) ? kpos[s1 - 1] + keep[s1 - 1] : c0;
    uint32_t a0 = (c1 > c0) ? accpos[c0] : 0u;
    uint32_t a1 = (c1 > c0) ? accpos[c1 - 1] + accf[c1 - 1] : 0u;
    meta[4 * r + 0] = c0;
    meta[4 * r + 1] = c1;
    meta[4 * r + 2] = a0;
    meta[4 * r + 3] = a1 - a0;
}

// Append accepted candidates in stream order up to each target.
// out[r*2 + {0: stream index+1 of the target-reaching rod, 1: density-accepted up to it}].
__global__ void k_append(const uint32_t* __restrict__ ntot, const uint8_t* __restrict__ state,
                         const uint32_t* __restrict__ creal, const uint32_t* __restrict__ accpos,
                         const uint32_t* __restrict__ meta, const uint32_t* __restrict__ rodoff,
                         const uint32_t* __restrict__ dcount, const Real* __restrict__ reals,
                         const float4* __restrict__ cpos, const float4* __restrict__ cdir,
                         const uint64_t* __restrict__ csidx, float4* __restrict__ pos, float4* __restrict__ dir,
                         uint64_t* __restrict__ sidx, uint64_t* __restrict__ out) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= *ntot || state[c] != ST_ACC) return;
    uint32_t r = creal[c];
    uint32_t rank = accpos[c] - meta[4 * r + 2];
    uint32_t have = dcount[r];
    uint32_t rem = reals[r].target - have;
    if (rank >= rem) return;
    uint32_t dst = rodoff[r] + have + rank;
    pos[dst] = cpos[c];
    dir[dst] = cdir[c];
    sidx[dst] = csidx[c];
    if (rank == rem - 1) {
        out[2 * r + 0] = csidx[c] + 1;
        out[2 * r + 1] = c - meta[4 * r + 0] + 1;
    }
}

// Rod cell list: counts.
__global__ void k_rod_count(uint32_t nslot, int R, const uint32_t* __restrict__ rodoff,
                            const uint32_t* __restrict__ dcount, const Real* __restrict__ reals,
                            const float4* __restrict__ pos, uint32_t* __restrict__ rcell,
                            uint32_t* __restrict__ ccount) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot) return;
    int r = find_real(rodoff, R, i);
    if (i - rodoff[r] >= dcount[r]) { rcell[i] = 0xffffffffu; return; }
    const Real& Re = reals[r];
    float4 p = pos[i];
    uint32_t cell = cell_of(Re, p.x, p.y, p.z);
    rcell[i] = cell;
    atomicAdd(&ccount[cell], 1u);
}

__global__ void k_rod_scatter(uint32_t nslot, const uint32_t* __restrict__ rcell, const uint32_t* __restrict__ start,
                              uint32_t* __restrict__ cursor, const float4* __restrict__ pos,
                              const float4* __restrict__ dir, float4* __restrict__ spos, float4* __restrict__ sdir,
                              uint32_t* __restrict__ sid) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot) return;
    uint32_t cell = rcell[i];
    if (cell == 0xffffffffu) return;
    uint32_t q = start[cell] + atomicAdd(&cursor[cell], 1u);
    spos[q] = pos[i];
    sdir[q] = dir[i];
    sid[q] = i;
}

// ---------------------------------------------------------------------------
// Host orchestration.
// ---------------------------------------------------------------------------
static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

nf_status Engine::cuda_fail(cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? NF_ERR_ALLOC : NF_ERR_CUDA;
}

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

cudaEvent_t Engine::tev() {
    cudaEvent_t e = nullptr;
    if (!evpool.empty()) { e = evpool.back(); evpool.pop_back(); }
    else cudaEventCreate(&e);
    return e;
}

// Folds recorded event pairs into per-kernel totals (synchronises the stream).
nf_status Engine::tresolve() {
    NF_CK(cudaStreamSynchronize(st));
    for (auto& k : kt) {
        for (auto& pr : k.ev) {
            float ms = 0;
            if (pr.first && pr.second) NF_CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
            k.ms += ms;
            if (pr.first) evpool.push_back(pr.first);
            if (pr.second) evpool.push_back(pr.second);
        }
        k.ev.clear();
    }
    return NF_OK;
}

__global__ void k_gather_pd(uint32_t n, const uint32_t* __restrict__ ntot, const uint32_t* __restrict__ perm,
                            const float4* __restrict__ pos, const float4* __restrict__ dir,
                            float4* __restrict__ opos, float4* __restrict__ odir) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t m = ntot ? *ntot : n;
    if (q >= m) return;
    uint32_t i = perm[q];
    opos[q] = pos[i];
    odir[q] = dir[i];
}

// Work list of one pair sweep: probes binned by pstart against targets binned
// by tstart, with the periodic flags of the stage (0 generation, 1 contacts).
nf_status Engine::ensure_pinned(size_t bytes) {
    if (bytes <= hpin_cap) return NF_OK;
    if (hpin) cudaFreeHost(hpin);
    hpin = nullptr;
    hpin_cap = 0;
    ++g_allocs;
    NF_CK(cudaMallocHost(reinterpret_cast<void**>(&hpin), bytes));
    hpin_cap = bytes;
    return NF_OK;
}

nf_status Engine::build_items(const uint32_t* pstart, const uint32_t* tstart, int stage, uint64_t np, uint64_t nt,
                              int ring) {
    const size_t n27 = (size_t)ncell * kRows;
    NF_CK(icnt.ensure(n27 + 1));
    NF_CK(ioff.ensure(n27 + 1));
    // Items of evenly spread probes and targets, with a quarter of headroom; a
    // work list that still overflows is grown and its pass redone.
    const double guess = 25.0 * ((double)np / kWC + ncell) * (1.0 + 5.0 * (double)nt / ((double)ncell * kSeg)) * 1.25;
    it_cap = std::max(it_cap, (size_t)std::min(guess, 4.0e8));
    NF_CK(items.ensure(it_cap));
    NF_LAUNCH(k_item_count, grid_for(n27 + 1, 256), 256, 0, st)(ncell, R, celloff.p, dreal.p, stage, ring, pstart,
                                                                 tstart, icnt.p);
    NF_CK(cudaGetLastError());
    nf_status s = scan_u32(icnt.p, ioff.p, n27 + 1);
    if (s != NF_OK) return s;
    // pairs per warp: 1 while pairs are few enough to give each its own warp
    const size_t per = n27 <= ((size_t)1 << 20) ? 1 : 32;
    NF_LAUNCH(k_item_fill, grid_for((n27 + per - 1) / per * 32, 256), 256, 0, st)(ncell, R, celloff.p, dreal.p, stage, ring, pstart, tstart, ioff.p,
                                                           items.p, (uint32_t)items.cap, ctr.p + C_ITEMS, (uint32_t)per);
    NF_CK(cudaGetLastError());
    return NF_OK;
}

// Exclusive scan of up to kSmallScan values in one block: each thread sums a
// contiguous run, the block scans the run totals, each thread writes its run.
// Reads each value before writing its own slot, so in == out is allowed.
constexpr size_t kSmallScan = 1 << 13;

__global__ void __launch_bounds__(1024) k_scan_small(const uint32_t* in, uint32_t* out, uint32_t n) {
    __shared__ uint32_t wsum[32];
    const uint32_t per = (n + 1023u) / 1024u;
    const uint32_t b = threadIdx.x * per, e = min(n, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += in[i];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t t = wsum[lane], ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += v;
        }
        wsum[lane] = ti - t;  // exclusive prefix of the warp totals
    }
    __syncthreads();
    uint32_t run = wsum[w] + incl - sum;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t v = in[i];
        out[i] = run;
        run += v;
    }
}

// Object sources of the tube registrations: placed rods of every realisation
// (slots beyond a realisation's count take no part), and the round's
// candidates still alive (compact ids, so the entries follow stream order).
struct TubeRodSrc {
    const uint32_t* rodoff;
    const uint32_t* dcount;
    int R;
    const float4* pos;
    const float4* dir;
    const uint32_t* dfirst;  // per realisation: first rod taken (null: 0)
    __device__ bool operator()(uint32_t i, int* r, float4* p, float4* c) const {
        const int q = find_real(rodoff, R, i);
        if (i - rodoff[q] >= dcount[q]) return false;
        if (dfirst && i - rodoff[q] < dfirst[q]) return false;
        *r = q;
        *p = pos[i];
        *c = dir[i];
        return true;
    }
    __device__ void geom(uint32_t i, float4* p, float4* c) const {
        *p = pos[i];
        *c = dir[i];
    }
};
struct TubeCandSrc {
    const uint32_t* creal;
    const float4* cpos;
    const float4* cdir;
    const uint8_t* state;
    __device__ bool operator()(uint32_t i, int* r, float4* p, float4* c) const {
        if (state[i] != ST_ALIVE) return false;
        *r = (int)creal[i];
        *p = cpos[i];
        *c = cdir[i];
        return true;
    }
    __device__ void geom(uint32_t i, float4* p, float4* c) const {
        *p = cpos[i];
        *c = cdir[i];
    }
};

nf_status Engine::tube_register_rods(int stage, bool room) {
    TubeRodSrc src{rodoff.p, dcount.p, R, pos.p, dir.p, nullptr};
    trod_append = false;
    // room for the rods still to come: growth (target - count) / count of each
    // realisation; none while some realisation has under a fifth of its
    // target (the room would be most of the registration)
    std::vector<float> g(R);
    for (int r = 0; room && r < R; ++r) {
        const double c = (double)count[r], t = (double)hreal[r].target;
        g[r] = (float)(t > c ? (t - c) / std::max(c, 1.0) : 0.0);
        if (g[r] > 4.0f) room = false;
    }
    trod_room = room;
    if (!room)
        return tube_register(*this, (uint32_t)rod_slots, nullptr, stage, src, trod_start, trod_cur, trod_ent, trod_pos,
                             trod_dir);
    // the cell counts then sit in trod_cur
    NF_CK(trod_grow.ensure(R));
    NF_CK(cudaMemcpyAsync(trod_grow.p, g.data(), sizeof(float) * R, cudaMemcpyHostToDevice, st));
    nf_status s = tube_register(*this, (uint32_t)rod_slots, nullptr, stage, src, trod_start, trod_cur, trod_ent,
                                trod_pos, trod_dir, trod_grow.p);  // g: a pageable copy, read in the call
    if (s != NF_OK) return s;
    trod_nreg = count;
    return NF_OK;
}

// The rods appended since the registration (rods trod_nreg[r] .. count[r] of
// each realisation) into the room of their cells: no count pass, no scan, no
// read-back; a cell without room counts in C_TROD_OVF (read back with the
// candidates' registration, which then registers all rods again).
nf_status Engine::tube_append_rods() {
    NF_CK(trod_dnreg.ensure(R));
    NF_CK(cudaMemcpyAsync(trod_dnreg.p, trod_nreg.data(), sizeof(uint32_t) * R, cudaMemcpyHostToDevice, st));
    NF_CK(cudaMemsetAsync(ctr.p + C_TROD_OVF, 0, sizeof(unsigned long long), st));
    TubeRodSrc src{rodoff.p, dcount.p, R, pos.p, dir.p, trod_dnreg.p};
    if (rod_slots) {
        auto kapp = k_treg<TubeRodSrc, 2>;
        NF_LAUNCH(kapp, (unsigned)((rod_slots + kRegTPB - 1) / kRegTPB), kRegTPB, 0, st)(
            (uint32_t)rod_slots, nullptr, dreal.p, 0, src, trod_cur.p, trod_start.p, trod_ent.p, trod_pos.p,
            trod_dir.p, 0u, ctr.p + C_TROD_OVF);
        NF_CK(cudaGetLastError());
    }
    trod_nreg = count;
    trod_append = false;
    return NF_OK;
}

nf_status Engine::tube_register_cands(uint64_t slots, const uint32_t* ntot, bool /*alive_only*/,
                                      const unsigned long long* extra, unsigned long long* extra_out) {
    TubeCandSrc src{creal.p, cpos.p, cdir.p, state.p};
    return tube_register(*this, (uint32_t)slots, ntot, 0, src, tcnd_start, tcnd_cur, tcnd_ent, tcnd_pos, tcnd_dir,
                         nullptr, extra, extra_out);
}

nf_status Engine::tube_items(const uint32_t* pstart, const uint32_t* tstart, const uint32_t* pcnt,
                              const uint32_t* tcnt, bool pack) {
    const uint32_t nseg = (ntcell + 31u) / 32u;
    // every item holds at least one probe entry, so the probe registration's
    // size bounds the items but where a cell's targets need several segments
    // (one more item per 128 targets of a cell beyond its first segment;
    // 1/64 of the targets is the allowance, and an overflow, counted in
    // C_ITEMS, redoes the stage with more room)
    const size_t nprobe = pstart == trod_start.p ? trod_total : tcnd_total;
    const size_t ntarget = tstart == trod_start.p ? trod_total : tcnd_total;
    tit_cap = std::max(tit_cap, nprobe + ntarget / 64 + 4096);
    NF_CK(icnt.ensure((size_t)nseg + 1));
    NF_CK(tioff.ensure((size_t)nseg + 1));
    NF_CK(titems.ensure(tit_cap));
    tit_nseg = nseg;
    const unsigned g = (unsigned)std::max<size_t>(1, std::min<size_t>(((size_t)nseg * 32 + 255) / 256, (size_t)nsm * 64));
    auto kcount = k_titem<false>;
    auto kfill = k_titem<true>;
    NF_LAUNCH(kcount, g, 256, 0, st)(ntcell, pack ? 1 : 0, toffs.p, R, pstart, tstart, pcnt, tcnt, icnt.p, nullptr,
                                     nullptr, 0u, nullptr);
    NF_CK(cudaGetLastError());
    nf_status s = scan_u32(icnt.p, tioff.p, (size_t)nseg + 1);
    if (s != NF_OK) return s;
    NF_LAUNCH(kfill, g, 256, 0, st)(ntcell, pack ? 1 : 0, toffs.p, R, pstart, tstart, pcnt, tcnt, nullptr, tioff.p,
                                    titems.p, (uint32_t)titems.cap, ctr.p + C_ITEMS);
    NF_CK(cudaGetLastError());
    return NF_OK;
}

nf_status Engine::tube_compact_cands() {
    NF_CK(tcnd_cnt.ensure((size_t)ntcell + 1));
    const unsigned blocks = (unsigned)std::min<size_t>(((size_t)ntcell + 7) / 8, (size_t)nsm * 16);
    NF_LAUNCH(k_treg_compact, std::max(1u, blocks), 256, 0, st)(ntcell, tcnd_start.p, tcnd_cnt.p, tcnd_ent.p,
                                                                 tcnd_pos.p, tcnd_dir.p, state.p,
                                                                 (uint8_t)ST_ALIVE);
    NF_CK(cudaGetLastError());
    return NF_OK;
}

nf_status Engine::scan_u32(const uint32_t* in, uint32_t* out, size_t n) {
    if (n <= kSmallScan) {
        NF_LAUNCH(k_scan_small, 1, 1024, 0, st)(in, out, (uint32_t)n);
        NF_CK(cudaGetLastError());
        return NF_OK;
    }
    g_launches += 2;  // DeviceScan: tile-state init + scan
    size_t bytes = 0;
    NF_CK(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int)n, st));
    NF_CK(cubtmp.ensure(bytes));
    NF_CK(cub::DeviceScan::ExclusiveSum(cubtmp.p, bytes, in, out, (int)n, st));
    return NF_OK;
}

uint64_t Engine::total_rods() const {
    uint64_t t = 0;
    for (uint32_t c : count) t += c;
    return t;
}

nf_status Engine::init(const nf_params* params, int n, const std::vector<const float*>& meshes) {
    R = n;
    prm.assign(params, params + n);
    NF_CK(cudaGetDevice(&dev));
    NF_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    hmesh.assign(n, {});
    for (int r = 0; r < n; ++r) {
        const nf_params& p = prm[r];
        if (meshes.size() > (size_t)r && meshes[r]) {
            size_t m = (size_t)p.mesh_ext[0] * p.mesh_ext[1] * p.mesh_ext[2];
            hmesh[r].assign(meshes[r], meshes[r] + m);
        }
    }
    count.assign(n, 0);
    knext.assign(n, 0);
    drawn.assign(n, 0);
    dens_acc.assign(n, 0);
    rounds_r.assign(n, 0);
    NF_CK(ctr.ensure(C_NCTR));
    return NF_OK;
}

nf_status Engine::set_density(int r, int nx, int ny, int nz, const float* values) {
    if (r < 0 || r >= R) return NF_ERR_PARAM;
    prm[r].mesh_ext[0] = nx;
    prm[r].mesh_ext[1] = ny;
    prm[r].mesh_ext[2] = nz;
    hmesh[r].assign(values, values + (size_t)nx * ny * nz);
    mesh_dirty = true;
    return NF_OK;
}

void Engine::release() {
    DBuf<float4>* f4[] = {&pos, &dir, &spos, &sdir, &cpos, &cdir, &gpos, &gdir, &vpf, &vdf, &apos, &adir};
    for (auto* b : f4) b->release();
    DBuf<uint32_t>* u32[] = {&inrod, &ieI, &ieJ, &ivals, &ivals2, &inew, &igid, &islot, &icnt, &ioff, &celloff, &vcell, &vperm, &vstart, &vcur, &aperm, &astart,
                             &dcount, &rodoff, &rstart, &rcursor, &sid, &coff, &keep, &kpos, &ccount,
                             &cstart, &ccursor, &cperm, &creal, &ccell, &ccnt, &clist, &accf, &accpos,
                             &meta, &u32tmp, &rcnt, &rpos, &rcur, &cI, &cJ, &creal2, &eflag, &parent,
                             &cflag, &aidx, &rowp, &col, &deg, &ecnt, &eoff, &elist};
    for (auto* b : u32) b->release();
    DBuf<uint64_t>* u64[] = {&sidx, &kbeg, &csidx};
    for (auto* b : u64) b->release();
    ikeys.release(); ikeys2.release();
    DBuf<double>* d64[] = {&ct0, &ct1, &cD, &cG, &cS, &vsrc, &vsnk, &volt, &val64, &diag64, &bvec, &xvec, &cgred,
                           &cdiag, &chain64, &valC64, &diagC64, &cdiagC, &bvecC, &acG, &acC, &acchi, &int_t, &ieG, &iseg_l};
    for (auto* b : d64) b->release();
    if (hpin) cudaFreeHost(hpin);
    hpin = nullptr;
    hpin_cap = 0;
    dreal.release(); mesh.release(); state.release(); ctr.release(); cubtmp.release(); items.release();
    vdbl.release();
    rec.release(); rec2.release(); recn.release(); cimg.release();
    val32.release(); diag32.release(); chain32.release(); cgbuf.release();
}

nf_status Engine::rebuild_cells() {
    NF_CK(cudaMemsetAsync(ccount.p, 0, sizeof(uint32_t) * (ncell + 1), st));
    NF_CK(u32tmp.ensure(rod_slots + 1));
    if (rod_slots) {
        NF_LAUNCH(k_rod_count, grid_for(rod_slots, 256), 256, 0, st)((uint32_t)rod_slots, R, rodoff.p, dcount.p, dreal.p,
                                                              pos.p, u32tmp.p, ccount.p);
        NF_CK(cudaGetLastError());
    }
    nf_status s = scan_u32(ccount.p, rstart.p, ncell + 1);
    if (s != NF_OK) return s;
    NF_CK(cudaMemsetAsync(rcursor.p, 0, sizeof(uint32_t) * (ncell + 1), st));
    if (rod_slots) {
        NF_LAUNCH(k_rod_scatter, grid_for(rod_slots, 256), 256, 0, st)((uint32_t)rod_slots, u32tmp.p, rstart.p, rcursor.p,
                                                                pos.p, dir.p, spos.p, sdir.p, sid.p);
        NF_CK(cudaGetLastError());
    }
    cells_valid = true;
    trod_stage = -1;  // the tube registrations of the rods are stale
    return NF_OK;
}

// Sets up grids, uploads meshes and realisation descriptors, sizes rod storage.
static nf_status setup_reals(Engine& E) {
    std::vector<uint32_t> mesh_off(E.R, 0);
    size_t mtot = 0;
    for (int r = 0; r < E.R; ++r) { mesh_off[r] = (uint32_t)mtot; mtot += E.hmesh[r].size(); }
    cudaError_t e = cudaSuccess;
    if (E.mesh_dirty || E.mesh.cap < mtot + 1) {
        e = E.mesh.ensure(mtot + 1);
        if (e != cudaSuccess) return E.cuda_fail(e, "mesh alloc");
    }
    if (E.mesh_dirty && mtot) {  // one copy through the pinned host buffer
        nf_status ps = E.ensure_pinned(mtot * sizeof(float));
        if (ps != NF_OK) return ps;
        float* stage = reinterpret_cast<float*>(E.hpin);
        for (int r = 0; r < E.R; ++r)
            if (!E.hmesh[r].empty()) std::memcpy(stage + mesh_off[r], E.hmesh[r].data(), E.hmesh[r].size() * sizeof(float));
        e = cudaMemcpyAsync(E.mesh.p, stage, mtot * sizeof(float), cudaMemcpyHostToDevice, E.st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(E.st);  // the staging buffer is reused later
        if (e != cudaSuccess) return E.cuda_fail(e, "mesh upload");
    }
    E.mesh_dirty = false;
    E.hreal.resize(E.R);
    uint32_t coffs = 0;
    uint64_t roff = 0, toffs = 0;
    std::vector<uint32_t> hrodoff(E.R + 1);
    for (int r = 0; r < E.R; ++r) {
        const nf_params& p = E.prm[r];
        int mn[3] = {p.mesh_ext[0], p.mesh_ext[1], p.mesh_ext[2]};
        const float* dm = E.hmesh[r].empty() ? nullptr : E.mesh.p + mesh_off[r];
        Real Re = make_real(p, dm, mn, stage_reach(p));
        Re.cell_off = coffs;
        Re.ncell = (uint32_t)(Re.n[0] * Re.n[1] * Re.n[2]);
        coffs += Re.ncell;
        Re.toff = (uint32_t)toffs;
        toffs += Re.tube ? Re.tncell : 0;
        if (toffs > 0xfffffff0ull) { E.err = "too many tube cells"; return NF_ERR_PARAM; }
        int64_t tgt = target_count(p);
        if (tgt < 0 || tgt > 0x7fffffff) { E.err = "target count out of range"; return NF_ERR_PARAM; }
        Re.target = (uint32_t)tgt;
        Re.rod_off = (uint32_t)roff;
        hrodoff[r] = (uint32_t)roff;
        roff += Re.target;
        if (roff > 0xffffff00ull) { E.err = "too many rods"; return NF_ERR_PARAM; }
        E.hreal[r] = Re;
    }
    hrodoff[E.R] = (uint32_t)roff;
    E.ncell = coffs;
    E.ntcell = (uint32_t)toffs;
    // the tube sweeps run when every realisation has a tube grid
    E.tube = E.ntcell > 0;
    for (int r = 0; r < E.R; ++r) E.tube = E.tube && E.hreal[r].tube;
    E.rod_slots = roff;
#define NF_CKS(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return E.cuda_fail(e_, #x); } while (0)
    std::vector<uint32_t> hcelloff(E.R + 1);
    for (int r = 0; r < E.R; ++r) hcelloff[r] = E.hreal[r].cell_off;
    hcelloff[E.R] = E.ncell;
    if (E.tube) {
        std::vector<uint32_t> ht(E.R + 1);
        for (int r = 0; r < E.R; ++r) ht[r] = E.hreal[r].toff;
        ht[E.R] = E.ntcell;
        NF_CKS(E.toffs.ensure(E.R + 1));
        NF_CKS(cudaMemcpyAsync(E.toffs.p, ht.data(), sizeof(uint32_t) * (E.R + 1), cudaMemcpyHostToDevice, E.st));
    }
    NF_CKS(E.celloff.ensure(E.R + 1));
    NF_CKS(cudaMemcpyAsync(E.celloff.p, hcelloff.data(), sizeof(uint32_t) * (E.R + 1), cudaMemcpyHostToDevice, E.st));
    NF_CKS(E.dreal.ensure(E.R));
    NF_CKS(cudaMemcpyAsync(E.dreal.p, E.hreal.data(), sizeof(Real) * E.R, cudaMemcpyHostToDevice, E.st));
    NF_CKS(E.rodoff.ensure(E.R + 1));
    NF_CKS(cudaMemcpyAsync(E.rodoff.p, hrodoff.data(), sizeof(uint32_t) * (E.R + 1), cudaMemcpyHostToDevice, E.st));
    NF_CKS(E.pos.ensure(roff + 1));
    NF_CKS(E.dir.ensure(roff + 1));
    NF_CKS(E.sidx.ensure(roff + 1));
    NF_CKS(E.spos.ensure(roff + 1));
    NF_CKS(E.sdir.ensure(roff + 1));
    NF_CKS(E.sid.ensure(roff + 1));
    NF_CKS(E.dcount.ensure(E.R));
    NF_CKS(E.rstart.ensure(E.ncell + 1));
    NF_CKS(E.rcursor.ensure(E.ncell + 1));
    NF_CKS(E.ccount.ensure(E.ncell + 1));
    NF_CKS(E.cstart.ensure(E.ncell + 1));
    NF_CKS(E.ccursor.ensure(E.ncell + 1));
#undef NF_CKS
    return NF_OK;
}

nf_status Engine::setup() { return setup_reals(*this); }

__global__ void k_stream_dump(const Real* __restrict__ reals, uint64_t k0, uint64_t n, float* __restrict__ out) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p, d;
    float u, rho;
    candidate(reals[0], k0 + i, &p, &d, &u, &rho);
    float* o = out + 10 * i;
    o[0] = p.x; o[1] = p.y; o[2] = p.z; o[3] = d.x; o[4] = d.y; o[5] = d.z;
    o[6] = p.w; o[7] = d.w; o[8] = u; o[9] = rho;
}

nf_status Engine::stream_dump(uint64_t k0, uint64_t n, float* host10) {
    nf_status s = setup_reals(*this);
    if (s != NF_OK) return s;
    DBuf<float> o;
    NF_CK(o.ensure(10 * n + 1));
    if (n) NF_LAUNCH(k_stream_dump, grid_for(n, 256), 256, 0, st)(dreal.p, k0, n, o.p);
    NF_CK(cudaGetLastError());
    NF_CK(cudaMemcpyAsync(host10, o.p, sizeof(float) * 10 * n, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    o.release();
    return NF_OK;
}

// Replace realisation 0's rods (e.g. read from output.bin); the target becomes n.
nf_status Engine::inject(size_t n, const float4* hpos, const float4* hdir, const uint64_t* hsidx) {
    if (R != 1) { err = "rods can be set on a single-realisation handle only"; return NF_ERR_STATE; }
    prm[0].n_target = (int64_t)n;
    nf_status s = setup_reals(*this);
    if (s != NF_OK) return s;
    if (n) {
        NF_CK(cudaMemcpyAsync(pos.p, hpos, sizeof(float4) * n, cudaMemcpyHostToDevice, st));
        NF_CK(cudaMemcpyAsync(dir.p, hdir, sizeof(float4) * n, cudaMemcpyHostToDevice, st));
        if (hsidx) NF_CK(cudaMemcpyAsync(sidx.p, hsidx, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, st));
        else NF_CK(cudaMemsetAsync(sidx.p, 0xff, sizeof(uint64_t) * n, st));
    }
    count.assign(1, (uint32_t)n);
    knext.assign(1, 0);
    drawn.assign(1, 0);
    dens_acc.assign(1, 0);
    NF_CK(cudaMemcpyAsync(dcount.p, count.data(), sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    s = rebuild_cells();
    if (s != NF_OK) return s;
    contacts_valid = false;
    solve_valid = false;
    int_valid = false;
    std::memset(&gst, 0, sizeof(gst));
    gst.accepted = n;
    gst.target = n;
    gst.target_reached = 1;
    NF_CK(cudaStreamSynchronize(st));
    return NF_OK;
}

// Candidates of one round over all realisations at most (~300 B of device
// memory per candidate slot).
constexpr uint64_t kRoundSlotCap = 1ull << 24;

nf_status Engine::generate() {
    nf_status s = setup_reals(*this);
    if (s != NF_OK) return s;
    cudaEvent_t e0, e1;
    NF_CK(cudaEventCreate(&e0));
    NF_CK(cudaEventCreate(&e1));
    NF_CK(cudaEventRecord(e0, st));
    std::fill(count.begin(), count.end(), 0u);
    std::fill(knext.begin(), knext.end(), 0ull);
    std::fill(drawn.begin(), drawn.end(), 0ull);
    std::fill(dens_acc.begin(), dens_acc.end(), 0ull);
    std::fill(rounds_r.begin(), rounds_r.end(), 0);
    NF_CK(cudaMemsetAsync(dcount.p, 0, sizeof(uint32_t) * R, st));
    NF_CK(cudaMemsetAsync(ctr.p, 0, sizeof(unsigned long long) * C_NCTR, st));
    s = rebuild_cells();
    if (s != NF_OK) return s;
    contacts_valid = false;
    solve_valid = false;
    int_valid = false;
    // Adaptive generation: epochs of the candidate stream (a round never
    // crosses a boundary); laws refit and rods thinned at boundaries; the
    // candidates of an epoch snap to the n_old rods present when it began.
    s = laws_reset();
    if (s != NF_OK) return s;
    const bool adapt = adaptive();
    ad_epochs = ad_refits = ad_thinned = ad_snapped = 0;
    const uint64_t epoch_len = adapt ? (prm[0].epoch_candidates > 0 ? (uint64_t)prm[0].epoch_candidates
                                                                      : std::max<uint64_t>(1024, hreal[0].target))
                                     : 0;
    uint64_t epoch_begun = ~0ull;
    uint32_t epoch_count0 = 0, n_old = 0;

    // Round sizing statistics.
    std::vector<double> p_dens(R), alive_max(R);
    for (int r = 0; r < R; ++r) {
        const nf_params& p = prm[r];
        double mean = p.density_default, peak = 1.0;
        if (!hmesh[r].empty()) {
            double sm = 0, mx = 0;
            for (float v : hmesh[r]) { sm += v; mx = std::max(mx, (double)v); }
            mean = sm / hmesh[r].size();
            peak = mean > 0 ? std::max(1.0, mx / mean) : 1.0;
        }
        p_dens[r] = std::min(1.0, std::max(mean, 1e-3));
        double lmax, amax;
        size_bounds(p, &lmax, &amax);
        double V = (double)p.box[0] * p.box[1] * p.box[2];
        double vex = 0.5 * M_PI * lmax * lmax * (2 * amax + p.sep) + 1e-12;
        // ~8 expected in-round conflicts per survivor at the density peak
        // (a conflict list overflow redoes the round at half size)
        alive_max[r] = std::max(4096.0, 8.0 * V / (vex * peak));
    }
    std::vector<uint32_t> hcoff(R + 1);
    std::vector<uint64_t> hkbeg(R);
    std::vector<uint64_t> c_round(R);
    std::vector<double> last_rate(R, 1.0);  // accepted / drawn in the last round
    double scale = 1.0;
    int rounds = 0, redone = 0;
    const int max_rounds = 100000;
    for (; rounds < max_rounds; ++rounds) {
        if (adapt && count[0] < hreal[0].target && knext[0] < prm[0].n_candidates && knext[0] % epoch_len == 0 &&
            knext[0] != epoch_begun) {
            if (knext[0] > 0) {
                s = epoch_boundary(knext[0] / epoch_len - 1, count[0] - epoch_count0);
                if (s != NF_OK) return s;
            }
            epoch_begun = knext[0];
            epoch_count0 = count[0];
            n_old = count[0];
            ++ad_epochs;
        }
        uint64_t slots = 0;
        int active = 0;
        for (int r = 0; r < R; ++r) {
            const nf_params& p = prm[r];
            uint64_t c = 0;
            uint32_t tgt = hreal[r].target;
            if (count[r] < tgt && knext[r] < p.n_candidates) {
                // Acceptance per candidate: the density acceptance before the
                // first round, then the last round's own rate (the rate only
                // falls as the box fills, so the cumulative rate would
                // overestimate it). Rounds draw round_overshoot (1.5 by default)
                // times the expected need: extra candidates cost sweep work, a
                // short round costs a round.
                const double acc_rate = rounds_r[r] > 0 ? last_rate[r] : p_dens[r];
                const double over = p.round_overshoot > 0 ? (double)p.round_overshoot : 1.5;
                double want = (tgt - count[r]) / std::max(acc_rate, 1e-6) * over + 256;
                // Survivors of the old-rod test per round: at most alive_max
                // (bounds the conflict lists) and at most the target count
                // (in-round conflict work grows with the square of the
                // survivors; measured on 256 realisations, a cap of the target
                // beats half of it by 15 %).
                const double grow = std::max(4096.0, (double)tgt);
                double amax_c = std::min(alive_max[r], grow) / std::max(acc_rate, 1e-6);
                double cr = std::min(want, p.round_candidates > 0 ? (double)p.round_candidates : amax_c) * scale;
                c = (uint64_t)std::max(64.0, cr);
                c = std::min<uint64_t>(c, p.n_candidates - knext[r]);
                c = std::min<uint64_t>(c, 1u << 24);
                if (adapt) c = std::min<uint64_t>(c, epoch_len - knext[r] % epoch_len);
                // clusterisation lists: candidates x older rods within half a
                // rod length (a few hundred at jamming) stay below 2^32
                if (adapt && p.clust_flag) c = std::min<uint64_t>(c, 1u << 20);
                ++active;
            }
            c_round[r] = c;
            hcoff[r] = (uint32_t)slots;
            hkbeg[r] = knext[r];
            slots += c;
        }
        if (slots > kRoundSlotCap) {  // bound the round's memory: scale every realisation down
            const double f = (double)kRoundSlotCap / (double)slots;
            slots = 0;
            for (int r = 0; r < R; ++r) {
                if (c_round[r]) c_round[r] = std::max<uint64_t>(std::min<uint64_t>(64, c_round[r]),
                                                                (uint64_t)(c_round[r] * f));
                hcoff[r] = (uint32_t)slots;
                slots += c_round[r];
            }
        }
        hcoff[R] = (uint32_t)slots;
        if (!active) break;
        // Buffers.
        NF_CK(coff.ensure(R + 1));
        NF_CK(kbeg.ensure(R));
        NF_CK(keep.ensure(slots + 1));
        NF_CK(kpos.ensure(slots + 1));
        NF_CK(cpos.ensure(slots));
        NF_CK(cdir.ensure(slots));
        NF_CK(csidx.ensure(slots));
        NF_CK(creal.ensure(slots));
        NF_CK(ccell.ensure(slots));
        NF_CK(cperm.ensure(slots));
        NF_CK(gpos.ensure(slots));
        NF_CK(gdir.ensure(slots));
        NF_CK(apos.ensure(slots));
        NF_CK(adir.ensure(slots));
        NF_CK(aperm.ensure(slots));
        NF_CK(astart.ensure(ncell + 1));
        NF_CK(state.ensure(slots));
        NF_CK(ccnt.ensure(slots));
        NF_CK(clist.ensure(slots * kConflictCap));
        NF_CK(accf.ensure(slots + 1));
        NF_CK(accpos.ensure(slots + 1));
        NF_CK(meta.ensure(4 * R));
        NF_CK(recn.ensure(2 * R + 2));
        NF_CK(cudaMemcpyAsync(coff.p, hcoff.data(), sizeof(uint32_t) * (R + 1), cudaMemcpyHostToDevice, st));
        NF_CK(cudaMemcpyAsync(kbeg.p, hkbeg.data(), sizeof(uint64_t) * R, cudaMemcpyHostToDevice, st));
        const unsigned gs = grid_for(slots, 256);
        tstart(KT_STREAM);
        NF_LAUNCH(k_stream_keep, gs, 256, 0, st)(dreal.p, R, coff.p, kbeg.p, (uint32_t)slots, keep.p);
        NF_CK(cudaGetLastError());
        tstop(KT_STREAM);
        NF_CK(cudaMemsetAsync(keep.p + slots, 0, sizeof(uint32_t), st));
        s = scan_u32(keep.p, kpos.p, slots + 1);  // kpos[slots] = compacted total
        if (s != NF_OK) return s;
        uint32_t* ntot = kpos.p + slots;
        // the tube sweeps read the compact candidates directly; the stencil
        // sweeps need them binned by cell
        const bool tube_round = tube && !adapt;
        if (!tube_round) NF_CK(cudaMemsetAsync(ccount.p, 0, sizeof(uint32_t) * (ncell + 1), st));
        const size_t shc = !tube_round && ncell <= kShCells ? sizeof(uint32_t) * ncell : 0;
        const unsigned gb = grid_for(slots, kBinTPB);
        NF_LAUNCH(k_compact, gb, kBinTPB, shc, st)(dreal.p, R, coff.p, kbeg.p, (uint32_t)slots, keep.p, kpos.p, cpos.p,
                                                   cdir.p, csidx.p, creal.p, tube_round ? nullptr : ccell.p,
                                                   ccount.p, state.p, ncell);
        NF_CK(cudaGetLastError());
        const bool clustered = adapt && prm[0].clust_flag && n_old > 0;
        if (clustered) {
            s = clusterize(slots, ntot, n_old);
            if (s != NF_OK) return s;
        }
        if (!tube_round) {
            s = scan_u32(ccount.p, cstart.p, ncell + 1);
            if (s != NF_OK) return s;
            NF_CK(cudaMemsetAsync(ccursor.p, 0, sizeof(uint32_t) * (ncell + 1), st));
            NF_LAUNCH(k_bin, gb, kBinTPB, 2 * shc, st)((uint32_t)slots, ntot, ccell.p, cstart.p, ccursor.p, cperm.p, ncell);
            NF_CK(cudaGetLastError());
            // Cell-sorted candidate copy and the chunk table of this round.
            NF_LAUNCH(k_gather_pd, gs, 256, 0, st)((uint32_t)slots, ntot, cperm.p, cpos.p, cdir.p, gpos.p, gdir.p);
            NF_CK(cudaGetLastError());
        }
        // The old-rod test runs in phases when the grid has outer stencil rows
        // and the round is heavy: every candidate against the centre row
        // (dy = dz = 0: the 5 cells nearest along x, 1/25 of the volume, where
        // most rejected candidates find their first hit), then only the
        // survivors, packed densely again, against the four rows next to it,
        // then the four inner corner rows, then the outer rows. A warp pays for
        // its dead lanes until its item ends; the packing keeps the lanes busy.
        // Same decisions as one pass; each further pass costs a binning, a work
        // list and two launches (~0.1 ms), repaid once candidates x rods passes
        // ~1e10 (jammed box: old_test 84.5 -> 31.5 ms per step with three
        // phases against two split at the inner ring; four phases save another
        // 1.5 % there and 3.6 % on the large box; five, with the outer rows
        // split, no more).
        bool outer_rows = false;
        double work = 0;
        for (int r = 0; r < R; ++r) {
            outer_rows |= c_round[r] && hreal[r].S > 1;
            work += (double)c_round[r] * (double)count[r];
        }
        const double two_work = prm[0].two_phase_work != 0 ? prm[0].two_phase_work : 1e10;
        const bool phased = outer_rows && two_work >= 0 && work > two_work;
        NF_CK(cudaMemsetAsync(ctr.p + C_ITEMS, 0, sizeof(unsigned long long), st));
        if (!tube) {
            s = build_items(cstart.p, rstart.p, 0, slots, total_rods(), phased ? 3 : 0);
            if (s != NF_OK) return s;
        }
        const unsigned xg = (unsigned)(4 * nsm);
        // first guess (8 B a slot, a fresh handle's first rounds must not
        // overflow it); grown and the round redone on overflow
        xq_cap = std::max(xq_cap, (size_t)(slots / 2));
        NF_CK(xq.ensure(xq_cap));
        NF_CK(xq2.ensure(xq_cap));
        NF_CK(cudaMemsetAsync(ctr.p + C_XQ_OLD, 0, 2 * sizeof(unsigned long long), st));
        // Survivors of the candidates in cell order (aperm / apos / adir, CSR astart).
        auto bin_survivors = [&]() -> nf_status {
            NF_CK(cudaMemsetAsync(ccursor.p, 0, sizeof(uint32_t) * (ncell + 1), st));
            NF_LAUNCH(k_alive_count, gs, 256, 0, st)((uint32_t)slots, ntot, cperm.p, state.p, ccell.p, ccursor.p);
            NF_CK(cudaGetLastError());
            nf_status s2 = scan_u32(ccursor.p, astart.p, ncell + 1);
            if (s2 != NF_OK) return s2;
            NF_CK(cudaMemsetAsync(ccursor.p, 0, sizeof(uint32_t) * (ncell + 1), st));
            NF_LAUNCH(k_alive_bin, gs, 256, 0, st)((uint32_t)slots, ntot, cperm.p, state.p, ccell.p, astart.p,
                                                   ccursor.p, gpos.p, gdir.p, aperm.p, apos.p, adir.p);
            NF_CK(cudaGetLastError());
            return NF_OK;
        };
        tstart(KT_OLD);
        bool cands_registered = false;  // the tube registration of this round's candidates
        if (tube && total_rods() > 0) {
            // tube grid: the kept candidates against the placed rods that share
            // a cell. The rods' registration (stage 0) leaves room in every
            // cell; the rods of the rounds after it are appended, and a full
            // registration follows only when a cell runs out of room.
            bool appended = false;
            if (trod_stage == 0 && trod_append && trod_room) {
                s = tube_append_rods();
                if (s != NF_OK) return s;
                appended = true;
            } else if (trod_stage != 0 || trod_append) {
                s = tube_register_rods(0, tube_round);
                if (s != NF_OK) return s;
                trod_stage = 0;
            }
            unsigned long long rod_ovf = 0;
            s = tube_register_cands(slots, ntot, true, appended ? ctr.p + C_TROD_OVF : nullptr, &rod_ovf);
            if (s != NF_OK) return s;
            if (rod_ovf) {
                s = tube_register_rods(0, true);
                if (s != NF_OK) return s;
            }
            cands_registered = true;
            s = tube_items(tcnd_start.p, trod_start.p, nullptr, trod_cur.p, true);
            if (s != NF_OK) return s;
            NF_LAUNCH(k_tube_old, persistent_grid(k_tube_old), kTPB, 0, st)(dreal.p, R, toffs.p, titem_count(),
                                                    (uint32_t)titems.cap, titems.p, tcnd_start.p, trod_start.p,
                                                    trod_cur.p, tcnd_ent.p, tcnd_pos.p, tcnd_dir.p,
                                                    trod_ent.p, trod_pos.p, trod_dir.p, state.p, xq.p, xq.cap, ctr.p);
            NF_CK(cudaGetLastError());
            NF_LAUNCH(k_old_exact, xg, 256, 0, st)(dreal.p, xq.p, nullptr, ctr.p + C_XQ_OLD, xq.cap, cpos.p, cdir.p,
                                                   creal.p, pos.p, dir.p, state.p, ctr.p);
        } else if (total_rods() > 0) {
            NF_LAUNCH(k_old_tiles, persistent_grid(k_old_tiles), kTPB, 0, st)(dreal.p, item_count(), (uint32_t)items.cap, items.p, cperm.p, gpos.p,
                                                    gdir.p, spos.p, sdir.p, state.p, xq.p, xq.cap, ctr.p);
            NF_CK(cudaGetLastError());
            NF_LAUNCH(k_old_exact, xg, 256, 0, st)(dreal.p, xq.p, nullptr, ctr.p + C_XQ_OLD, xq.cap, cpos.p, cdir.p,
                                                   creal.p, spos.p, sdir.p, state.p, ctr.p);
        }
        NF_CK(cudaGetLastError());
        for (int ring : {5, 6, 2}) {  // the survivors against the next inner rows, the inner corners, the outer rows
            if (!phased || tube) break;
            NF_CK(cudaMemcpyAsync(ctr.p + C_XQ_MARK, ctr.p + C_XQ_OLD, sizeof(unsigned long long),
                                  cudaMemcpyDeviceToDevice, st));
            s = bin_survivors();
            if (s != NF_OK) return s;
            s = build_items(astart.p, rstart.p, 0, slots, total_rods(), ring);
            if (s != NF_OK) return s;
            NF_LAUNCH(k_old_tiles, persistent_grid(k_old_tiles), kTPB, 0, st)(dreal.p, item_count(), (uint32_t)items.cap, items.p, aperm.p, apos.p,
                                                    adir.p, spos.p, sdir.p, state.p, xq.p, xq.cap, ctr.p);
            NF_CK(cudaGetLastError());
            NF_LAUNCH(k_old_exact, xg, 256, 0, st)(dreal.p, xq.p, ctr.p + C_XQ_MARK, ctr.p + C_XQ_OLD, xq.cap,
                                                   cpos.p, cdir.p, creal.p, spos.p, sdir.p, state.p, ctr.p);
            NF_CK(cudaGetLastError());
        }
        tstop(KT_OLD);
        const uint32_t* scnt = nullptr;  // per-cell survivor counts of a compacted registration
        if (tube) {  // the survivors on the tube grid: the round's registration compacted, or registered
            if (cands_registered) {
                s = tube_compact_cands();
                scnt = tcnd_cnt.p;
            } else {
                s = tube_register_cands(slots, ntot, true);
            }
            if (s != NF_OK) return s;
            s = tube_items(tcnd_start.p, tcnd_start.p, scnt, scnt, true);
            if (s != NF_OK) return s;
        } else {
            s = bin_survivors();
            if (s != NF_OK) return s;
            s = build_items(astart.p, astart.p, 0, slots, slots);
            if (s != NF_OK) return s;
        }
        NF_CK(cudaMemsetAsync(ctr.p + C_OVERFLOW, 0, sizeof(unsigned long long), st));
        NF_CK(cudaMemsetAsync(ccnt.p, 0, sizeof(uint32_t) * slots, st));
        tstart(KT_CONF);
        if (tube) {
            NF_CK(xqc.ensure(xq2.cap));
            NF_LAUNCH(k_tube_conf, persistent_grid(k_tube_conf), kTPB, 0, st)(dreal.p, R, toffs.p, titem_count(),
                                                    (uint32_t)titems.cap, titems.p, tcnd_start.p, scnt,
                                                    tcnd_ent.p, tcnd_pos.p, tcnd_dir.p,
                                                    ccnt.p, clist.p, xq2.p, xqc.p, xq2.cap, ctr.p);
        } else {
            NF_LAUNCH(k_conf_tiles, persistent_grid(k_conf_tiles), kTPB, 0, st)(dreal.p, item_count(), (uint32_t)items.cap, items.p, aperm.p, apos.p,
                                                 adir.p, ccnt.p, clist.p, xq2.p, xq2.cap, ctr.p);
        }
        NF_CK(cudaGetLastError());
        NF_LAUNCH(k_conf_exact, xg, 256, 0, st)(dreal.p, xq2.p, tube ? xqc.p : nullptr, ctr.p + C_XQ_CONF, xq2.cap,
                                                cpos.p, cdir.p, creal.p, ccnt.p, clist.p, ctr.p);
        NF_CK(cudaGetLastError());
        tstop(KT_CONF);
        // Resolution passes (chains are short), then the append, optimistic
        // until one read-back of the counters shows that every candidate was
        // decided; otherwise more passes and a fresh append (it is idempotent:
        // the device rod counts change only after the read-back).
        static_assert(C_UNDECIDED == C_OVERFLOW + 1 && C_ITEMS == C_XQ_OLD + 4, "read-back layout");
        uint64_t passes = 0;
        bool redo = false;
        // pinned read-back block: [0..1] overflow, undecided; [2..6] old queue,
        // conflict queue, (C_XQ, C_CERT), work items; then recn (2R u64), meta (4R u32)
        s = ensure_pinned(sizeof(unsigned long long) * (7 + 2 * (size_t)R) + sizeof(uint32_t) * 4 * (size_t)R);
        if (s != NF_OK) return s;
        unsigned long long* hv = reinterpret_cast<unsigned long long*>(hpin);
        uint64_t* hout = reinterpret_cast<uint64_t*>(hv + 7);
        uint32_t* hmeta = reinterpret_cast<uint32_t*>(hout + 2 * R);
        for (;;) {
            NF_CK(cudaMemsetAsync(ctr.p + C_UNDECIDED, 0, sizeof(unsigned long long), st));
            NF_LAUNCH(k_resolve, gs, 256, 0, st)(ntot, state.p, ccnt.p, clist.p, ctr.p, 16);
            NF_CK(cudaGetLastError());
            passes += 16;
            NF_LAUNCH(k_accflag, grid_for(slots + 1, 256), 256, 0, st)(ntot, (uint32_t)(slots + 1), state.p, accf.p);
            NF_CK(cudaGetLastError());
            s = scan_u32(accf.p, accpos.p, slots + 1);
            if (s != NF_OK) return s;
            NF_LAUNCH(k_meta, grid_for(R, 128), 128, 0, st)(R, coff.p, keep.p, kpos.p, accf.p, accpos.p, meta.p);
            NF_CK(cudaGetLastError());
            NF_CK(cudaMemsetAsync(recn.p, 0, sizeof(unsigned long long) * 2 * R, st));
            NF_LAUNCH(k_append, gs, 256, 0, st)(ntot, state.p, creal.p, accpos.p, meta.p, rodoff.p, dcount.p, dreal.p,
                                                cpos.p, cdir.p, csidx.p, pos.p, dir.p, sidx.p, (uint64_t*)recn.p);
            NF_CK(cudaGetLastError());
            NF_CK(cudaMemcpyAsync(&hv[0], ctr.p + C_OVERFLOW, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  st));
            NF_CK(cudaMemcpyAsync(&hv[2], ctr.p + C_XQ_OLD, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  st));
            NF_CK(cudaMemcpyAsync(hout, recn.p, sizeof(uint64_t) * 2 * R, cudaMemcpyDeviceToHost, st));
            NF_CK(cudaMemcpyAsync(hmeta, meta.p, sizeof(uint32_t) * 4 * R, cudaMemcpyDeviceToHost, st));
            NF_CK(cudaStreamSynchronize(st));
            if (!tube && hv[6] > items.cap) {  // work list too small: grow it and redo the round
                it_cap = (size_t)(hv[6] * 1.25) + 4096;
                redo = true;
                break;
            }
            if (tube && hv[6] > titems.cap) {
                tit_cap = (size_t)(hv[6] * 1.25) + 4096;
                redo = true;
                break;
            }
            if (hv[2] > xq.cap || hv[3] > xq2.cap) {  // exact queue too small: grow it and redo the round
                xq_cap = (size_t)(std::max(hv[2], hv[3]) * 1.25) + 1024;
                redo = true;
                break;
            }
            if (hv[0]) {  // too many in-round conflicts: redo the round with fewer candidates
                scale *= 0.5;
                if (scale < 1e-4) { err = "in-round conflict list overflow"; return NF_ERR_OVERFLOW; }
                redo = true;
                break;
            }
            if (!hv[1]) break;
            if (passes > 4096) { err = "conflict resolution did not converge"; return NF_ERR_TIMEOUT; }
        }
        if (redo) {
            --rounds;
            ++redone;
            continue;
        }
        bool any_new = false;
        {
            double nc = 0;
            for (int r = 0; r < R; ++r) nc += c_round[r] ? (double)(hmeta[4 * r + 1] - hmeta[4 * r + 0]) : 0.0;
            tbytes(KT_OLD, 33.0 * nc + 32.0 * (double)total_rods(), 0);
        }
        for (int r = 0; r < R; ++r) {
            if (!c_round[r]) continue;
            ++rounds_r[r];
            last_rate[r] = std::max(1e-7, (double)hmeta[4 * r + 3] / (double)c_round[r]);
            uint32_t rem = hreal[r].target - count[r];
            uint32_t got = std::min(hmeta[4 * r + 3], rem);
            uint32_t kept = hmeta[4 * r + 1] - hmeta[4 * r + 0];
            if (got) any_new = true;
            count[r] += got;
            if (count[r] == hreal[r].target && got == rem && rem > 0) {
                drawn[r] = hout[2 * r + 0];
                dens_acc[r] += hout[2 * r + 1];
            } else {
                dens_acc[r] += kept;
            }
            knext[r] += c_round[r];
            if (count[r] < hreal[r].target) drawn[r] = knext[r];
        }
        if (clustered) {  // snaps of the candidates this round consumed
            s = count_snaps(slots, ntot, drawn[0]);
            if (s != NF_OK) return s;
        }
        NF_CK(cudaMemcpyAsync(dcount.p, count.data(), sizeof(uint32_t) * R, cudaMemcpyHostToDevice, st));
        if (any_new) {
            if (tube_round) {  // the cell lists wait for the end of the generation
                cells_valid = false;
                trod_append = true;  // the new rods go into the room of the registration
            } else {
                s = rebuild_cells();
                if (s != NF_OK) return s;
            }
        }
        scale = std::min(1.0, scale * 2.0);
    }
    if (!cells_valid) {
        s = rebuild_cells();
        if (s != NF_OK) return s;
    }
    NF_CK(cudaEventRecord(e1, st));
    NF_CK(cudaEventSynchronize(e1));
    float ms = 0;
    NF_CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    unsigned long long hc[C_NCTR];
    NF_CK(cudaMemcpy(hc, ctr.p, sizeof(hc), cudaMemcpyDeviceToHost));
    if (hc[C_TUBE_OVF]) { err = "tube registration beyond its bound"; return NF_ERR_OVERFLOW; }
    std::memset(&gst, 0, sizeof(gst));
    for (int r = 0; r < R; ++r) {
        gst.candidates_drawn += drawn[r];
        gst.density_accepted += dens_acc[r];
        gst.accepted += count[r];
        gst.target += hreal[r].target;
    }
    gst.pair_tests = hc[C_PAIR_TESTS];
    gst.work_items = hc[C_G_ITEMS];
    gst.target_tiles = hc[C_G_TILES];
    gst.marked_pairs = hc[C_G_MARKED];
    gst.line_pairs = hc[C_G_LINE];
    gst.exact_evals = hc[C_EXACT];
    gst.fp32_would_flip = hc[C_FLIPS];
    gst.exact_evals = hc[C_EXACT];
    gst.rounds = rounds;
    gst.epochs = ad_epochs;
    gst.refits = ad_refits;
    gst.thinned = ad_thinned;
    gst.snapped = ad_snapped;
    gst.target_reached = gst.accepted == gst.target;
    gst.ms = ms;
    gst.tube_grid = tube ? 1 : 0;
    gst.redone_rounds = redone;
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
