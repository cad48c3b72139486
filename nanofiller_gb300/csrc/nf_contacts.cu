// nf_contacts.cu -- tunnelling-contact extraction, screening and electrode roles.
//
// Reference path replaced: collect_cunduct_data steps 1-5 (src/conductivity.cu:140-226)
// = get_contact_counts / get_contact_arrays (src/get_contact_arrays.cu:12-140) on
// core_cell_interact_kernel COUNT/RECORD (src/core_cell_interaction_kernel.cu:69-315),
// check_screened_contacts + generate_virt_inclusions + VIRTUAL_CHECK
// (src/conductivity.cu:430-528, inc/conductKernels.h:289-361,
// src/check_screened_Interactions.cu:12-70), sort_contacts_by_role
// (src/conductivity.cu:530-637), get_contact_distance / get_contact_surface
// (src/get_contact_data.cu:28-230).
//
// One sweep replaces COUNT + scan + RECORD: every contact found is appended to a
// record buffer (global atomic, sized from the previous count and re-run once
// if it overflows), then records are counting-sorted by their lower rod id and
// each rod's short run is ordered by (J, image). The pair rule is the
// reference's: rod I tests rods J > I of the 27 neighbour cells, J shifted by
// the cell's periodic image (upper triangle + image shift, :115, :249-259), so
// a rod never meets its own image (sameFLG, :253).
#include <algorithm>
#include <cmath>
#include <cstring>

#include <cub/device/device_radix_sort.cuh>

#include "nf_engine.cuh"
#include "nf_tiles.cuh"

namespace nf {

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

// ---------------------------------------------------------------------------
// Pair sweep: one (rod chunk, stencil offset) per block, neighbour rods staged
// in shared memory. Rod I considers rods J > I (upper triangle); pairs the FP32
// filter cannot rule out are queued (probe, target = sorted rod indices) and
// recorded by k_ct_exact from their FP64 evaluation.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kTPB, 6) k_ct_tiles(const Real* __restrict__ reals,
                                                   const uint32_t* __restrict__ nitems, uint32_t icap,
                                                   const Item* __restrict__ items,
                                                   const float4* __restrict__ spos, const float4* __restrict__ sdir,
                                                   const uint32_t* __restrict__ sid, unsigned long long* __restrict__ xq,
                                                   unsigned long long xcap, unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ WarpTile tiles[kW];
    __shared__ uint32_t tid_[kW][kWT];
    __shared__ float4 ppos[kW][32], pdir[kW][32];
    __shared__ int msp[kW][32];
    __shared__ uint32_t msm[kW][32];
    __shared__ uint16_t mq2[kW][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpTile& T = tiles[w];
    const float epc = 1e-6f;  // DEV_PRECISION (inc/definitions.h:5)
    unsigned long long tests = 0;
    const uint32_t n = min(*nitems, icap);
    const uint32_t stride = gridDim.x * kW;
    Item nxt = blockIdx.x * kW + w < n ? items[blockIdx.x * kW + w] : Item{0, 0, 0, 0};
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += stride) {
        const Item I = nxt;
        if (it + stride < n) nxt = items[it + stride];  // next item's descriptor in flight meanwhile
        uint32_t np, nt;
        int img[3];
        item_unpack(I, &np, &nt, img);
        const Real& Re = reals[I.real];
        const bool have = (uint32_t)lane < np;
        const uint32_t q = I.pfirst + lane;
        uint32_t i = 0xffffffffu;
        float4 pA = make_float4(0, 0, 0, 0), cA = pA;
        if (have) { i = sid[q]; pA = spos[q]; cA = sdir[q]; }
        __syncwarp();
        ppos[w][lane] = pA;
        pdir[w][lane] = cA;
        const float sx = img[0] * Re.L[0], sy = img[1] * Re.L[1], sz = img[2] * Re.L[2];
        const float ax = pA.x - sx, ay = pA.y - sy, az = pA.z - sz;
        const float hA2 = (pA.w * 0.5f + cA.w + epc + cA.w + Re.cut + epc) * 1.000002f + Re.slack;
        const float hAe = pA.w * 0.5f + cA.w + epc;
        const float hC = (cA.w + Re.cut + epc) * 1.000002f + Re.slack + 4e-6f * (1.0f + hA2);
        for (uint32_t b = 0; b < nt; b += kWT) {
            const uint32_t m = min((uint32_t)kWT, nt - b);
            if ((uint32_t)lane < m) {
                const uint32_t k = I.tfirst + b + lane;
                const float4 p = spos[k], c = sdir[k];
                T.l[lane] = p.w;
                T.p[lane] = make_float4(p.x, p.y, p.z, (p.w * 0.5f + c.w + epc + c.w) * 1.000002f);
                T.c[lane] = c;
                tid_[w][lane] = sid[k];
            } else {
                T.p[lane] = make_float4(kFar, kFar, kFar, 0.0f);
                tid_[w][lane] = 0u;
            }
            __syncwarp();
            uint32_t mask = 0, umask = 0;  // marked pairs; pairs with J > I
            if (have) {
                const uint32_t m8 = (m + 7u) & ~7u;
                for (uint32_t j0 = 0; j0 < m8; j0 += 8) {
#pragma unroll
                    for (uint32_t jj = 0; jj < 8; ++jj) {
                        const uint32_t j = j0 + jj;
                        const float4 tq = T.p[j];
                        const float bx = tq.x - ax, by = tq.y - ay, bz = tq.z - az;
                        const uint32_t bit = tid_[w][j] > i ? (1u << j) : 0u;  // each unordered pair once
                        umask |= bit;
                        if (capsule_near(bx, by, bz, cA.x, cA.y, cA.z, hAe, tq.w, hC)) mask |= bit;
                    }
                }
                tests += __popc(umask);
            }
            const uint32_t base = I.tfirst + b;
            auto keep = [&](int pl, int t) {
                const float4 dA = pdir[w][pl], tq = T.p[t], cB = T.c[t];
                const float4 pB = make_float4(tq.x, tq.y, tq.z, T.l[t]);
                return !line_far(ppos[w][pl], dA, pB, cB, sx, sy, sz, (cB.w + dA.w) + Re.cut + epc, Re.slack);
            };
            (void)for_marked_pairs(mask, lane, msp[w], msm[w], mq2[w], keep, [&](bool valid, int pl, int t) {
                if (!valid) return;
                const float4 qA = ppos[w][pl], dA = pdir[w][pl];
                const float4 tq = T.p[t], cB = T.c[t];
                const float4 pB = make_float4(tq.x, tq.y, tq.z, T.l[t]);
                const float thr = (cB.w + dA.w) + Re.cut + epc;
                if (maybe_near(qA, dA, pB, cB, sx, sy, sz, thr, epc, Re.slack))
                    xq_push(xq, xcap, &ctr[C_XQ], xq_pack(I.pfirst + pl, base + t, img));
            });
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_CT_PAIRS], tests);
}

__global__ void __launch_bounds__(256) k_ct_exact(const Real* __restrict__ reals, int R,
                                                  const uint32_t* __restrict__ rodoff,
                                                  const unsigned long long* __restrict__ xq,
                                                  const unsigned long long* __restrict__ count, unsigned long long xcap,
                                                  const float4* __restrict__ spos, const float4* __restrict__ sdir,
                                                  const uint32_t* __restrict__ sid, Rec* __restrict__ rec,
                                                  unsigned long long cap, unsigned long long* __restrict__ recn,
                                                  uint32_t* __restrict__ rcnt, unsigned long long* __restrict__ ctr) {
    const unsigned long long n = min(*count, xcap);
    const float epc = 1e-6f;
    unsigned long long exact = 0, flips = 0;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t q, p;
        int img[3];
        xq_unpack(xq[e], &q, &p, img);
        const uint32_t i = sid[q], j = sid[p];
        const Real& Re = reals[find_real(rodoff, R, i)];
        const float4 pA = spos[q], cA = sdir[q], pB = spos[p], cB = sdir[p];
        ++exact;
        const RodD a = rodd(pA, cA), b = rodd(pB, cB);
        double t0d, t1d, u0, u1, Dx;
        double d = ref_distance_d(a, b, img[0] * (double)Re.L[0], img[1] * (double)Re.L[1],
                                  img[2] * (double)Re.L[2], (double)epc, false, &t0d, &t1d, &u0, &u1, &Dx);
        bool h = d < thresh_d(a.a, b.a, 1.0, (double)Re.cut, (double)epc);
        const float thr = (cB.w + cA.w) + Re.cut + epc;
        if (ref_hit_f32(pA, cA, pB, cB, img[0] * Re.L[0], img[1] * Re.L[1], img[2] * Re.L[2], epc, thr, false) != h)
            ++flips;
        if (!h) continue;
        unsigned long long slot = atomicAdd(recn, 1ull);
        atomicAdd(&rcnt[i], 1u);
        if (slot < cap) {
            Rec x;
            x.i = i;
            x.j = j;
            x.img[0] = (int8_t)img[0];
            x.img[1] = (int8_t)img[1];
            x.img[2] = (int8_t)img[2];
            x.img[3] = 0;
            x.flags = 0;
            x.t0 = t0d; x.t1 = t1d; x.d = d; x.Dx = Dx; x.u0 = u0; x.u1 = u1;
            rec[slot] = x;
        }
    }
    warp_add_u64(&ctr[C_CT_EXACT], exact);
    warp_add_u64(&ctr[C_CT_FLIPS], flips);
}

// Contact sweep on the tube grid: rod I against rods J > I registered in the
// same tube cell (entries carry the image of each rod's copy); pairs the FP32
// filter cannot rule out are queued with their cell (rod ids, relative image).
// Marking: the line bound, then the capsule test (the hand-out then only
// checks the relative image).
__global__ void __launch_bounds__(kTPB, 7) k_tube_ct(const Real* __restrict__ reals, int R,
                                                  const uint32_t* __restrict__ toffs,
                                                  const uint32_t* __restrict__ nitems, uint32_t icap,
                                                  const TItem* __restrict__ items,
                                                  const uint32_t* __restrict__ start, const uint32_t* __restrict__ ent,
                                                  const float4* __restrict__ pos, const float4* __restrict__ dir,
                                                  unsigned long long* __restrict__ xq, uint32_t* __restrict__ xqc,
                                                  unsigned long long xcap, unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ TubeTile tiles[kW];
    __shared__ TubePack packs[kW];
    __shared__ float4 ppos[kW][32], pdir[kW][32];
    __shared__ uint32_t pid[kW][32], pim[kW][32], pcel[kW][32];
    __shared__ int msp[kW][32];
    __shared__ uint32_t msm[kW][32];
    __shared__ uint16_t mq2[kW][64];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    TubeTile& T = tiles[w];
    const float epc = 1e-6f;  // DEV_PRECISION (inc/definitions.h:5)
    unsigned long long tests = 0;
    const uint32_t n = min(*nitems, icap);
    const uint32_t stride = gridDim.x * kW;
    TItem nxt = blockIdx.x * kW + w < n ? items[blockIdx.x * kW + w] : TItem{0, 0, 0, 0};
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += stride) {
        const TItem I = nxt;
        if (it + stride < n) nxt = items[it + stride];
        const TubeLane L = tube_lane(I, lane, start, start, nullptr, nullptr, packs[w]);
        const uint32_t np = L.np, nt = L.nt;
        const Real& Re = reals[item_real(I.pfirst, I.cnt, I.cell, toffs, R)];
        const bool have = (uint32_t)lane < np;
        uint32_t i = 0xffffffffu, ip = 0;
        float4 pA = make_float4(0, 0, 0, 0), cA = pA;
        if (have) {
            const uint32_t e = ent[L.pe];
            i = e >> kTubeIdShift;
            ip = e & 63u;
            pA = pos[L.pe];
            cA = dir[L.pe];
        }
        __syncwarp();
        ppos[w][lane] = pA;
        pdir[w][lane] = cA;
        pid[w][lane] = i;
        pim[w][lane] = ip;
        pcel[w][lane] = L.cell;
        int ia[3];
        img_of(ip, ia);
        const float ax = pA.x + ia[0] * Re.L[0], ay = pA.y + ia[1] * Re.L[1], az = pA.z + ia[2] * Re.L[2];
        const float hA2 = (pA.w * 0.5f + cA.w + epc + cA.w + Re.cut + epc) * 1.000002f + Re.slack;
        const float hAe = pA.w * 0.5f + cA.w + epc;
        const float hC = (cA.w + Re.cut + epc) * 1.000002f + 2.0f * Re.slack + 4e-6f * (1.0f + hA2);
        const float errA = 4e-6f * (1.0f + hA2) + 2.0f * Re.slack;
        const float thA = (cA.w + Re.cut + epc) * 1.0002f;
        for (uint32_t b = 0; b < nt; b += kWT) {
            const uint32_t m = min((uint32_t)kWT, nt - b);
            // each pair once (probe and target entries are one list): tiles
            // before the item's probe chunk are left to the items whose chunk
            // they are; on the chunk's own tile (and in packed items, where
            // probe lane p is target slot p) a rod tests the next half of its
            // range, cyclically; tiles after the chunk are tested whole
            if (!L.packed && I.tfirst + b < I.pfirst) continue;
            const bool self = L.packed || I.tfirst + b == I.pfirst;
            if ((uint32_t)lane < m) {
                uint32_t tc;
                const uint32_t q = tube_target(I, L, packs[w], b, (uint32_t)lane, &tc);
                (void)tc;
                const uint32_t e = ent[q];
                const uint32_t k = e >> kTubeIdShift;
                const float4 p = pos[q], c = dir[q];
                int ib[3];
                img_of(e & 63u, ib);
                T.p[lane] = p;
                T.ps[lane] = make_float4(p.x + ib[0] * Re.L[0], p.y + ib[1] * Re.L[1], p.z + ib[2] * Re.L[2],
                                         (p.w * 0.5f + c.w + epc + c.w) * 1.000002f);
                T.c[lane] = c;
                T.id[lane] = k;
                T.im[lane] = e & 63u;
            } else {
                T.ps[lane] = make_float4(kFar, kFar, kFar, 0.0f);
                T.id[lane] = 0u;
            }
            __syncwarp();
            const uint32_t lo = L.packed ? L.tlo : 0u, len = L.packed ? L.tlen : m;
            const uint32_t xl = (uint32_t)lane - lo;
            const uint32_t nd = !self ? len : (len ? (len - 1u) / 2u + ((len & 1u) == 0u && xl < len / 2u) : 0u);
            uint32_t mask = 0;  // marked pairs
            if (have) {
                for (uint32_t u0 = 0; u0 < nd; u0 += 8) {
#pragma unroll
                    for (uint32_t jj = 0; jj < 8; ++jj) {
                        const uint32_t u = u0 + jj;
                        if (u < nd) {
                            uint32_t y = self ? xl + 1u + u : u;
                            if (y >= len) y -= len;
                            const uint32_t j = lo + y;
                            const float4 tq = T.ps[j];
                            const float bx = tq.x - ax, by = tq.y - ay, bz = tq.z - az;
                            const uint32_t bit = 1u << j;
                            const float4 cB = T.c[j];
                            const float nx = cA.y * cB.z - cA.z * cB.y;
                            const float ny = cA.z * cB.x - cA.x * cB.z;
                            const float nz = cA.x * cB.y - cA.y * cB.x;
                            const float nn = nx * nx + ny * ny + nz * nz;
                            const float nb = fabsf(nx * bx + ny * by + nz * bz) - fmaf(4e-6f, tq.w, errA);
                            const float thL = fmaf(cB.w, 1.0002f, thA);
                            const bool lfar = nn > 1e-4f && nb > 0.0f && nb * nb > thL * thL * nn;
                            if (!lfar && capsule_near(bx, by, bz, cA.x, cA.y, cA.z, hAe, tq.w, hC)) mask |= bit;
                        }
                    }
                }
                tests += nd;
            }
            auto keep = [&](int pl, int t) {
                int img[3];
                return rel_img(pim[w][pl], T.im[t], img);
            };
            (void)for_marked_pairs(mask, lane, msp[w], msm[w], mq2[w], keep, [&](bool valid, int pl, int t) {
                if (!valid) return;
                // the rod of the smaller id is the pair's first rod I
                const bool sw = T.id[t] < pid[w][pl];
                const float4 qA = sw ? T.p[t] : ppos[w][pl], dA = sw ? T.c[t] : pdir[w][pl];
                const float4 pB = sw ? ppos[w][pl] : T.p[t], cB = sw ? pdir[w][pl] : T.c[t];
                int img[3];
                rel_img(pim[w][pl], T.im[t], img);
                if (sw) {
                    img[0] = -img[0];
                    img[1] = -img[1];
                    img[2] = -img[2];
                }
                const float thr = (cB.w + dA.w) + Re.cut + epc;
                if (maybe_near(qA, dA, pB, cB, img[0] * Re.L[0], img[1] * Re.L[1], img[2] * Re.L[2], thr, epc,
                               Re.slack))
                    xq_push_cell(xq, xqc, xcap, &ctr[C_XQ],
                                 xq_pack(sw ? T.id[t] : pid[w][pl], sw ? pid[w][pl] : T.id[t], img), pcel[w][pl]);
            });
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_CT_PAIRS], tests);
}

// FP64 records of the tube sweep's queue; a pair found in several cells is
// recorded by the one that holds the midpoint of its two points.
__global__ void __launch_bounds__(256) k_ct_exact_tube(const Real* __restrict__ reals, int R,
                                                       const uint32_t* __restrict__ rodoff,
                                                       const unsigned long long* __restrict__ xq,
                                                       const uint32_t* __restrict__ xqc,
                                                       const unsigned long long* __restrict__ count,
                                                       unsigned long long xcap, const float4* __restrict__ pos,
                                                       const float4* __restrict__ dir, Rec* __restrict__ rec,
                                                       unsigned long long cap, unsigned long long* __restrict__ recn,
                                                       uint32_t* __restrict__ rcnt, unsigned long long* __restrict__ ctr) {
    const unsigned long long n = min(*count, xcap);
    const float epc = 1e-6f;
    unsigned long long exact = 0, flips = 0;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t i, j;
        int img[3];
        xq_unpack(xq[e], &i, &j, img);
        const Real& Re = reals[find_real(rodoff, R, i)];
        const float4 pA = pos[i], cA = dir[i], pB = pos[j], cB = dir[j];
        ++exact;
        const RodD a = rodd(pA, cA), b = rodd(pB, cB);
        const double sx = img[0] * (double)Re.L[0], sy = img[1] * (double)Re.L[1], sz = img[2] * (double)Re.L[2];
        double t0d, t1d, u0, u1, Dx;
        double d = ref_distance_d(a, b, sx, sy, sz, (double)epc, false, &t0d, &t1d, &u0, &u1, &Dx);
        bool h = d < thresh_d(a.a, b.a, 1.0, (double)Re.cut, (double)epc);
        if (h && !tube_claims_d(Re, Re.per_con, xqc[e], a, b, sx, sy, sz, t0d, t1d)) continue;
        const float thr = (cB.w + cA.w) + Re.cut + epc;
        if (ref_hit_f32(pA, cA, pB, cB, img[0] * Re.L[0], img[1] * Re.L[1], img[2] * Re.L[2], epc, thr, false) != h)
            ++flips;
        if (!h) continue;
        unsigned long long slot = atomicAdd(recn, 1ull);
        atomicAdd(&rcnt[i], 1u);
        if (slot < cap) {
            Rec x;
            x.i = i;
            x.j = j;
            x.img[0] = (int8_t)img[0];
            x.img[1] = (int8_t)img[1];
            x.img[2] = (int8_t)img[2];
            x.img[3] = 0;
            x.flags = 0;
            x.t0 = t0d; x.t1 = t1d; x.d = d; x.Dx = Dx; x.u0 = u0; x.u1 = u1;
            rec[slot] = x;
        }
    }
    warp_add_u64(&ctr[C_CT_EXACT], exact);
    warp_add_u64(&ctr[C_CT_FLIPS], flips);
}

__global__ void k_rec_scatter(uint32_t n, const Rec* __restrict__ rec, const uint32_t* __restrict__ rpos,
                              uint32_t* __restrict__ rcur, Rec* __restrict__ out) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    Rec x = rec[q];
    uint32_t dst = rpos[x.i] + atomicAdd(&rcur[x.i], 1u);
    out[dst] = x;
}

__device__ __forceinline__ bool rec_less(const Rec& a, const Rec& b) {
    if (a.j != b.j) return a.j < b.j;
    for (int d = 2; d >= 0; --d)
        if (a.img[d] != b.img[d]) return a.img[d] < b.img[d];
    return false;
}

// Order each rod's run by (J, image z, y, x): insertion sort (runs are short).
__global__ void k_rec_sort(uint32_t nslot, const uint32_t* __restrict__ rpos, const uint32_t* __restrict__ rcnt,
                           Rec* __restrict__ rec) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot) return;
    uint32_t b = rpos[i], n = rcnt[i];
    for (uint32_t a = 1; a < n; ++a) {
        Rec x = rec[b + a];
        uint32_t k = a;
        while (k > 0 && rec_less(x, rec[b + k - 1])) {
            rec[b + k] = rec[b + k - 1];
            --k;
        }
        rec[b + k] = x;
    }
}

// ---------------------------------------------------------------------------
// Screening: the segment between the two contact points (radius min(aI,aJ))
// is a virtual rod; the contact is dropped if any real rod crosses its body
// (if_intersects with separation 0, then body_intersect on the unclamped
// parameter along the virtual rod; src/core_cell_interaction_kernel.cu:141-146).
// k_virt builds the virtual rods (FP64 record + FP32 copy) and bins them by
// the cell of their centre wrapped into the box; k_scr_tiles tests them.
// ---------------------------------------------------------------------------
constexpr int kVD = 11;  // doubles per virtual rod: x y z cx cy cz l a, wrap shift x y z

__global__ void k_virt(int R, const uint32_t* __restrict__ rodoff, uint32_t nrec, const Rec* __restrict__ rec,
                       const float4* __restrict__ pos, const float4* __restrict__ dir,
                       const Real* __restrict__ reals, double* __restrict__ vd, float4* __restrict__ vpf,
                       float4* __restrict__ vdf, uint32_t* __restrict__ vcell, uint32_t* __restrict__ vcount) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrec) return;
    const Rec x = rec[q];
    const int r = find_real(rodoff, R, x.i);
    const Real& Re = reals[r];
    const RodD A = rodd(pos[x.i], dir[x.i]);
    const RodD B = rodd(pos[x.j], dir[x.j]);
    const double sh[3] = {x.img[0] * (double)Re.L[0], x.img[1] * (double)Re.L[1], x.img[2] * (double)Re.L[2]};
    const double p0[3] = {dadd(A.x, dmul(x.t0, A.cx)), dadd(A.y, dmul(x.t0, A.cy)), dadd(A.z, dmul(x.t0, A.cz))};
    const double p1[3] = {dadd(dadd(B.x, sh[0]), dmul(x.t1, B.cx)), dadd(dadd(B.y, sh[1]), dmul(x.t1, B.cy)),
                          dadd(dadd(B.z, sh[2]), dmul(x.t1, B.cz))};
    double vr[3], vc[3];
    for (int d = 0; d < 3; ++d) {
        vr[d] = dmul(dadd(p0[d], p1[d]), 0.5);
        vc[d] = dsub(p1[d], p0[d]);
    }
    double vl = dsqrt(dadd(dadd(dmul(vc[0], vc[0]), dmul(vc[1], vc[1])), dmul(vc[2], vc[2])));
    if (!(vl > 0)) { vcell[q] = 0xffffffffu; return; }
    double inv = ddiv(1.0, vl);
    for (int d = 0; d < 3; ++d) vc[d] = dmul(vc[d], inv);
    const double va = fmin(A.a, B.a);
    double vw[3];
    for (int d = 0; d < 3; ++d) {
        double xw = vr[d];
        if (Re.per_con & (1 << d)) {
            xw = fmod(xw, (double)Re.L[d]);
            if (xw < 0) xw = dadd(xw, (double)Re.L[d]);
        }
        vw[d] = xw;
    }
    double* o = vd + (size_t)kVD * q;
    o[0] = vr[0]; o[1] = vr[1]; o[2] = vr[2];
    o[3] = vc[0]; o[4] = vc[1]; o[5] = vc[2];
    o[6] = vl; o[7] = va;
    o[8] = dsub(vw[0], vr[0]); o[9] = dsub(vw[1], vr[1]); o[10] = dsub(vw[2], vr[2]);
    vpf[q] = make_float4((float)vr[0], (float)vr[1], (float)vr[2], (float)vl);
    vdf[q] = make_float4((float)vc[0], (float)vc[1], (float)vc[2], (float)va);
    const uint32_t cell = cell_of(Re, (float)vw[0], (float)vw[1], (float)vw[2]);
    vcell[q] = cell;
    atomicAdd(&vcount[cell], 1u);
}

__global__ void k_vbin(uint32_t n, const uint32_t* __restrict__ cellof, const uint32_t* __restrict__ start,
                       uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t cell = cellof[i];
    if (cell == 0xffffffffu) return;  // zero-length segment: never screened
    perm[start[cell] + atomicAdd(&cursor[cell], 1u)] = i;
}

__global__ void __launch_bounds__(kTPB) k_scr_tiles(const Real* __restrict__ reals,
                                                    const uint32_t* __restrict__ nitems, uint32_t icap,
                                                    const Item* __restrict__ items,
                                                    const uint32_t* __restrict__ vperm,
                                                    const double* __restrict__ vd, const float4* __restrict__ vpf,
                                                    const float4* __restrict__ vdf,
                                                    const float4* __restrict__ spos, const float4* __restrict__ sdir,
                                                    unsigned long long* __restrict__ xq, unsigned long long xcap,
                                                    unsigned long long* __restrict__ ctr) {
    __shared__ WarpTile tiles[kTPB / 32];
    // the chunk's virtual rods for the transposed loop (lanes on targets)
    __shared__ float4 vps[kTPB / 32][32], vds[kTPB / 32][32];
    __shared__ float vsh[kTPB / 32][32][3];
    __shared__ uint32_t vid[kTPB / 32][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpTile& T = tiles[w];
    const float epsf = 1e-6f;
    unsigned long long tests = 0;
    const uint32_t n = min(*nitems, icap);
    for (uint32_t it = blockIdx.x * (kTPB / 32) + w; it < n; it += gridDim.x * (kTPB / 32)) {
        const Item I = items[it];
        uint32_t np, nt;
        int img[3];
        item_unpack(I, &np, &nt, img);
        const Real& Re = reals[I.real];
        const bool have = (uint32_t)lane < np;
        const uint32_t id = have ? vperm[I.pfirst + lane] : 0u;
        float4 pV = make_float4(0, 0, 0, 0), cV = pV;
        float svf[3] = {0, 0, 0};
        if (have) {
            const double* o = vd + (size_t)kVD * id;
            for (int d = 0; d < 3; ++d) svf[d] = (float)dsub(o[8 + d], img[d] * (double)Re.L[d]);
            pV = vpf[id];
            cV = vdf[id];
            vps[w][lane] = pV;
            vds[w][lane] = cV;
            vsh[w][lane][0] = svf[0];
            vsh[w][lane][1] = svf[1];
            vsh[w][lane][2] = svf[2];
            vid[w][lane] = id;
        }
        __syncwarp();
        for (uint32_t b = 0; b < nt; b += kWT) {
            if (b + lane < nt) {
                T.p[lane] = spos[I.tfirst + b + lane];
                T.c[lane] = sdir[I.tfirst + b + lane];
            }
            __syncwarp();
            const uint32_t m = min((uint32_t)kWT, nt - b);
            if (np < m) {
                // fewer virtual rods than staged rods (contacts are sparse):
                // lane = rod, the warp walks the chunk's np virtual rods
                if ((uint32_t)lane < m) {
                    tests += np;
                    const float4 pR = T.p[lane], cR = T.c[lane];
                    for (uint32_t pi = 0; pi < np; ++pi) {
                        const float4 pv = vps[w][pi], cv = vds[w][pi];
                        const float thr = (cv.w + cR.w) + epsf;
                        if (maybe_near(pR, cR, pv, cv, vsh[w][pi][0], vsh[w][pi][1], vsh[w][pi][2], thr, epsf,
                                       Re.slack))
                            xq_push(xq, xcap, &ctr[C_XQ], xq_pack(vid[w][pi], I.tfirst + b + lane, img));
                    }
                }
            } else if (have) {
                tests += m;
                for (uint32_t j = 0; j < m; ++j) {
                    const float4 pR = T.p[j], cR = T.c[j];
                    const float thr = (cV.w + cR.w) + epsf;
                    if (!maybe_near(pR, cR, pV, cV, svf[0], svf[1], svf[2], thr, epsf, Re.slack)) continue;
                    xq_push(xq, xcap, &ctr[C_XQ], xq_pack(id, I.tfirst + b + j, img));
                }
            }
            __syncwarp();
        }
    }
    warp_add_u64(&ctr[C_SCR_PAIRS], tests);
}

// Screening on the tube grid: the virtual rods of one cell (probe entries)
// against the rods registered there (target entries); one lane per rod, the
// warp walks the cell's virtual rods (contacts are sparse). Virtual rods sit
// at their unwrapped centre; a pair's shift is the relative image of the
// virtual rod's copy.
__global__ void __launch_bounds__(kTPB) k_tube_scr(const Real* __restrict__ reals, int R,
                                                   const uint32_t* __restrict__ toffs,
                                                   const uint32_t* __restrict__ nitems, uint32_t icap,
                                                   const TItem* __restrict__ items, const uint32_t* __restrict__ vent,
                                                   const float4* __restrict__ vpf, const float4* __restrict__ vdf,
                                                   const uint32_t* __restrict__ rent, const float4* __restrict__ pos,
                                                   const float4* __restrict__ dir, unsigned long long* __restrict__ xq,
                                                   unsigned long long xcap, unsigned long long* __restrict__ ctr) {
    constexpr int kW = kTPB / 32;
    __shared__ float4 vps[kW][32], vds[kW][32];
    __shared__ uint32_t vid[kW][32], vim[kW][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float epsf = 1e-6f;
    unsigned long long tests = 0;
    const uint32_t n = min(*nitems, icap);
    for (uint32_t it = blockIdx.x * kW + w; it < n; it += gridDim.x * kW) {
        const TItem I = items[it];
        const uint32_t np = I.cnt & 63u, nt = (I.cnt >> 6) & 0xFFu;
        const Real& Re = reals[item_real(I.pfirst, I.cnt, I.cell, toffs, R)];
        if ((uint32_t)lane < np) {
            const uint32_t e = vent[I.pfirst + lane];
            const uint32_t id = e >> kTubeIdShift;
            vps[w][lane] = vpf[I.pfirst + lane];
            vds[w][lane] = vdf[I.pfirst + lane];
            vid[w][lane] = id;
            vim[w][lane] = e & 63u;
        }
        __syncwarp();
        for (uint32_t b = lane; b < nt; b += 32) {
            const uint32_t e = rent[I.tfirst + b];
            const uint32_t k = e >> kTubeIdShift, ir = e & 63u;
            const float4 pR = pos[I.tfirst + b], cR = dir[I.tfirst + b];
            tests += np;
            for (uint32_t pi = 0; pi < np; ++pi) {
                int img[3];
                if (!rel_img(ir, vim[w][pi], img)) continue;
                const float4 pv = vps[w][pi], cv = vds[w][pi];
                const float thr = (cv.w + cR.w) + epsf;
                if (maybe_near(pR, cR, pv, cv, img[0] * Re.L[0], img[1] * Re.L[1], img[2] * Re.L[2], thr, epsf,
                               Re.slack))
                    xq_push(xq, xcap, &ctr[C_XQ], xq_pack(vid[w][pi], k, img));
            }
        }
        __syncwarp();
    }
    warp_add_u64(&ctr[C_SCR_PAIRS], tests);
}

// FP64 screening decisions of the tube sweep's queue (virtual rod id, rod id,
// image of the virtual rod relative to the rod): k_scr_exact's test.
__global__ void __launch_bounds__(256) k_scr_exact_tube(const Real* __restrict__ reals, int R,
                                                        const uint32_t* __restrict__ rodoff,
                                                        const unsigned long long* __restrict__ xq,
                                                        const unsigned long long* __restrict__ count,
                                                        unsigned long long xcap, const double* __restrict__ vd,
                                                        const float4* __restrict__ pos, const float4* __restrict__ dir,
                                                        Rec* rec, unsigned long long* __restrict__ ctr) {
    const unsigned long long n = min(*count, xcap);
    const double eps = (double)1e-6f;
    unsigned long long exact = 0;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t id, p;
        int img[3];
        xq_unpack(xq[e], &id, &p, img);
        volatile uint32_t* vflag = &rec[id].flags;
        if (*vflag & 1u) continue;
        const Real& Re = reals[find_real(rodoff, R, rec[id].i)];
        const double* o = vd + (size_t)kVD * id;
        const RodD V{o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]};
        const RodD Rr = rodd(pos[p], dir[p]);
        ++exact;
        double u1, t0d, t1d, u0;
        double d = ref_distance_d(Rr, V, img[0] * (double)Re.L[0], img[1] * (double)Re.L[1],
                                  img[2] * (double)Re.L[2], eps, false, &t0d, &t1d, &u0, &u1, nullptr);
        bool h = d < thresh_d(Rr.a, V.a, 1.0, 0.0, eps);
        if (h && dsub(ddiv(V.l, 2.0), dabs(u1)) > dadd(V.a, eps)) atomicOr(&rec[id].flags, 1u);
    }
    warp_add_u64(&ctr[C_SCR_EXACT], exact);
}

__global__ void __launch_bounds__(256) k_scr_exact(const Real* __restrict__ reals, int R,
                                                   const uint32_t* __restrict__ rodoff,
                                                   const unsigned long long* __restrict__ xq,
                                                   const unsigned long long* __restrict__ count, unsigned long long xcap,
                                                   const double* __restrict__ vd, const float4* __restrict__ spos,
                                                   const float4* __restrict__ sdir, Rec* rec,
                                                   unsigned long long* __restrict__ ctr) {
    const unsigned long long n = min(*count, xcap);
    const double eps = (double)1e-6f;
    unsigned long long exact = 0;
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < n;
         e += (unsigned long long)gridDim.x * blockDim.x) {
        uint32_t id, p;
        int img[3];
        xq_unpack(xq[e], &id, &p, img);
        volatile uint32_t* vflag = &rec[id].flags;
        if (*vflag & 1u) continue;
        const Real& Re = reals[find_real(rodoff, R, rec[id].i)];
        const double* o = vd + (size_t)kVD * id;
        const RodD V{o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]};
        double sv[3];
        for (int d = 0; d < 3; ++d) sv[d] = dsub(o[8 + d], img[d] * (double)Re.L[d]);
        const RodD Rr = rodd(spos[p], sdir[p]);
        ++exact;
        double u1, t0d, t1d, u0;
        double d = ref_distance_d(Rr, V, sv[0], sv[1], sv[2], eps, false, &t0d, &t1d, &u0, &u1, nullptr);
        bool h = d < thresh_d(Rr.a, V.a, 1.0, 0.0, eps);
        if (h && dsub(ddiv(V.l, 2.0), dabs(u1)) > dadd(V.a, eps)) atomicOr(&rec[id].flags, 1u);
    }
    warp_add_u64(&ctr[C_SCR_EXACT], exact);
}

// ---------------------------------------------------------------------------
// Contact area, surf_to_cylinder_capped (inc/intersect/intersect_cylinder_capped.h:204-293)
// evaluated in FP64 for rod A and rod B shifted by sh.
// ---------------------------------------------------------------------------
__device__ double dot3(const double* u, const double* w) {
    return dadd(dadd(dmul(u[0], w[0]), dmul(u[1], w[1])), dmul(u[2], w[2]));
}

__device__ double contact_area(const RodD& A, const RodD& B, const double sh[3], double Dtt_x, double t1u,
                               double t2u, double rlim) {
    const double PIv = 3.141593;
    double l1 = A.l, l2 = B.l, a1 = A.a, a2 = B.a;
    double c1[3] = {A.cx, A.cy, A.cz}, c2[3] = {B.cx, B.cy, B.cz};
    double r1[3] = {A.x, A.y, A.z};
    double r2[3] = {dadd(B.x, sh[0]), dadd(B.y, sh[1]), dadd(B.z, sh[2])};
    double sg = copysign(1.0, dot3(c1, c2));
    double c2p[3] = {dmul(c2[0], sg), dmul(c2[1], sg), dmul(c2[2], sg)};
    double dr1 = 0.0, dr2 = 0.0;
    double h1 = fmax(dsub(dsub(Dtt_x, a2), rlim), 0.0);
    double h2 = fmax(dsub(dsub(Dtt_x, a1), rlim), 0.0);
    if (h1 <= a1) dr1 = dmul(a1, dsqrt(dsub(1.0, dmul(ddiv(h1, a1), ddiv(h1, a1)))));
    if (h2 <= a2) dr2 = dmul(a2, dsqrt(dsub(1.0, dmul(ddiv(h2, a2), ddiv(h2, a2)))));
    double dr = fmin(dr1, dr2);
    double S = dmul(dmul(PIv, dr), dr);
    double t1 = t1u, t2 = t2u;
    double d = dot3(c1, c2p);
    double sng = dsqrt(fmax(dsub(1.0, dmul(d, d)), 0.0));
    double hl1 = ddiv(l1, 2.0), hl2 = ddiv(l2, 2.0);
    if (dabs(t1) < dsub(hl1, a1) && dabs(t2) < dsub(hl2, a2)) {
        double ax1[3] = {dadd(c1[0], c2p[0]), dadd(c1[1], c2p[1]), dadd(c1[2], c2p[2])};
        double n1 = dsqrt(dot3(ax1, ax1));
        double in1 = ddiv(1.0, n1);
        for (int i = 0; i < 3; ++i) ax1[i] = dmul(ax1[i], in1);
        double csg = dsqrt(fmax(dsub(1.0, dmul(sng, sng)), 0.0));
        double sngh = dsqrt(ddiv(dsub(1.0, csg), 2.0));
        double t2p = copysign(t2, dot3(c1, c2));
        double dt0p = (sngh > 1e-6 ? ddiv(dr2, sngh) : hl1);
        double dt0m = dt0p;
        double qv[3];
        for (int i = 0; i < 3; ++i) qv[i] = dadd(r1[i], dmul(c1[i], dsub(hl1, t1)));
        double dt1p = dot3(qv, ax1);
        for (int i = 0; i < 3; ++i) qv[i] = dadd(r1[i], dmul(c1[i], dsub(-hl1, t1)));
        double dt1m = dabs(dot3(qv, ax1));
        for (int i = 0; i < 3; ++i) qv[i] = dadd(r2[i], dmul(c2p[i], dsub(hl2, t2p)));
        double dt2p = dot3(qv, ax1);
        for (int i = 0; i < 3; ++i) qv[i] = dadd(r2[i], dmul(c2p[i], dsub(-hl2, t2p)));
        double dt2m = dabs(dot3(qv, ax1));
        double Ap = fmax(dr, fmin(dt0p, fmin(dt1p, dt2p)));
        double Am = fmax(dr, fmin(dt0m, fmin(dt1m, dt2m)));
        S = fmax(S, dmul(dmul(dmul(0.5, PIv), dr), dadd(Ap, Am)));
    }
    if ((sng <= ddiv(fmax(a1, a2), fmin(l1, l2))) && (dabs(t1) <= dadd(hl1, a1) || dabs(t2) <= dadd(hl2, a2))) {
        double b[3] = {dsub(r2[0], r1[0]), dsub(r2[1], r1[1]), dsub(r2[2], r1[2])};
        double cb1 = dot3(c1, b), cb2 = dot3(c2, b);
        double t1a = copysign(hl1, cb1), t1b = dmul(-1.0, copysign(hl1, cb1));
        double t2a = copysign(hl2, cb2), t2b = dmul(-1.0, copysign(hl2, cb2));
        double qv[3];
        for (int i = 0; i < 3; ++i) qv[i] = dadd(r1[i], dmul(c1[i], t1a));
        double t1ac = dot3(qv, c1);
        for (int i = 0; i < 3; ++i) qv[i] = dadd(r1[i], dmul(c1[i], t1b));
        double t1bc = dot3(qv, c1);
        for (int i = 0; i < 3; ++i) qv[i] = dadd(dadd(b[i], r1[i]), dmul(c2[i], t2a));
        double t2ac = dot3(qv, c1);
        for (int i = 0; i < 3; ++i) qv[i] = dadd(dadd(b[i], r1[i]), dmul(c2[i], t2b));
        double t2bc = dot3(qv, c1);
        double p1c = cb1 > 0 ? fmin(t1ac, t2ac) : fmax(t1ac, t2ac);
        double p2c = cb1 > 0 ? fmax(t1bc, t2bc) : fmin(t1bc, t2bc);
        S = fmax(S, dmul(dmul(dabs(dsub(p2c, p1c)), 2.0), dr));
    }
    return S;
}

__device__ __forceinline__ double tunnel_g(const Real& Re, double gap) {
    double ge = gap > Re.dc ? gap : Re.dc;
    return Re.G0 * exp(-(ge - Re.dc) / Re.lambda);
}

// Per-realisation counts of unscreened / screened records. With buffer-layer
// electrodes (faxis >= 0) a kept record whose partner is an image across the
// field axis is not internal: it becomes one sink and one source contact
// (xf = 1; cnt[2R + 2r], cnt[2R + 2r + 1]).
__global__ void k_rec_count(int R, const uint32_t* __restrict__ rodoff, uint32_t nrec, const Rec* __restrict__ rec,
                            int faxis, uint32_t* __restrict__ keepf, uint32_t* __restrict__ xf,
                            uint32_t* __restrict__ cnt /* 4R */) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrec) return;
    const Rec& x = rec[q];
    int r = find_real(rodoff, R, x.i);
    bool scr = x.flags & 1u;
    const bool cross = !scr && faxis >= 0 && x.img[faxis] != 0;
    keepf[q] = (scr || cross) ? 0u : 1u;
    if (xf) xf[q] = cross ? 1u : 0u;
    if (cross) {
        atomicAdd(&cnt[2 * R + 2 * r], 1u);
        atomicAdd(&cnt[2 * R + 2 * r + 1], 1u);
    } else {
        atomicAdd(&cnt[2 * r + (scr ? 1 : 0)], 1u);
    }
}

// Buffer-layer electrode contacts of the cross records: the rod whose partner
// image lies below the box (img < 0 from i's side, > 0 from j's side) touches
// the source layer, the other rod the sink layer. Keys (rod, partner) for a
// stable sort; values the record index.
__global__ void k_buf_emit(uint32_t nrec, const Rec* __restrict__ rec, const uint32_t* __restrict__ xf,
                           const uint32_t* __restrict__ xpos, int faxis, uint32_t nx,
                           unsigned long long* __restrict__ key, uint32_t* __restrict__ val) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrec || !xf[q]) return;
    const Rec& x = rec[q];
    const uint32_t k = xpos[q];
    const bool below = x.img[faxis] < 0;  // j's image below: i touches the source layer
    const uint32_t src = below ? x.i : x.j, snk = below ? x.j : x.i;
    key[k] = ((unsigned long long)snk << 32) | (below ? x.i : x.j);            // sink list [0, nx)
    val[k] = q;
    key[nx + k] = ((unsigned long long)src << 32) | (below ? x.j : x.i);       // source list [nx, 2 nx)
    val[nx + k] = q;
}

// Final sink or source block of the buffer-layer contacts, from the sorted
// (rod, partner) list: realisation r's entries start at start[r].
__global__ void k_final_buf(uint32_t n, const unsigned long long* __restrict__ key, const uint32_t* __restrict__ val,
                            const Rec* __restrict__ rec, int R, const uint32_t* __restrict__ rodoff,
                            const uint32_t* __restrict__ start, const unsigned long long* __restrict__ base,
                            uint32_t elec_id, const Real* __restrict__ reals, const float4* __restrict__ pos,
                            const float4* __restrict__ dir, uint32_t* __restrict__ oI, uint32_t* __restrict__ oJ,
                            double* __restrict__ ot0, double* __restrict__ ot1, double* __restrict__ oD,
                            double* __restrict__ oG, double* __restrict__ oS, int8_t* __restrict__ oimg,
                            uint32_t* __restrict__ oreal) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const Rec x = rec[val[p]];
    const uint32_t rod = (uint32_t)(key[p] >> 32);
    const int r = find_real(rodoff, R, rod);
    const Real& Re = reals[r];
    const unsigned long long dst = base[r] + (p - start[r]);
    const bool iside = rod == x.i;
    const RodD A = rodd(pos[x.i], dir[x.i]);
    const RodD B = rodd(pos[x.j], dir[x.j]);
    oI[dst] = rod;
    oJ[dst] = elec_id;
    ot0[dst] = iside ? x.t0 : x.t1;
    ot1[dst] = iside ? x.t1 : x.t0;
    oD[dst] = x.d;
    oG[dst] = tunnel_g(Re, dsub(dsub(x.d, A.a), B.a));
    const double sh[3] = {x.img[0] * (double)Re.L[0], x.img[1] * (double)Re.L[1], x.img[2] * (double)Re.L[2]};
    oS[dst] = contact_area(A, B, sh, x.Dx, x.u0, x.u1, (double)Re.cut);
    for (int d = 0; d < 3; ++d) oimg[3 * dst + d] = (int8_t)(iside ? x.img[d] : -x.img[d]);
    oreal[dst] = (uint32_t)r;
}

// Electrode flags per rod slot: plane electrodes at x_f = 0 (source) and x_f = L_f (sink).
__global__ void k_elec(uint32_t nslot, int R, const uint32_t* __restrict__ rodoff, const uint32_t* __restrict__ dcount,
                       const Real* __restrict__ reals, const float4* __restrict__ pos, const float4* __restrict__ dir,
                       uint32_t* __restrict__ fsnk, uint32_t* __restrict__ fsrc, double* __restrict__ esnk /* D,t */,
                       double* __restrict__ esrc, uint32_t* __restrict__ cnt /* 2R: snk, src */) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot) return;
    int r = find_real(rodoff, R, i);
    const Real& Re = reals[r];
    fsnk[i] = 0;
    fsrc[i] = 0;
    if (i - rodoff[r] >= dcount[r] || Re.field_axis < 0) return;
    const RodD A = rodd(pos[i], dir[i]);
    const int f = Re.field_axis;
    const double cf = f == 0 ? A.cx : (f == 1 ? A.cy : A.cz);
    const double rf = f == 0 ? A.x : (f == 1 ? A.y : A.z);
    const double half = ddiv(A.l, 2.0);
    const double tlo = cf > 0 ? -half : half, thi = -tlo;
    const double zlo = dadd(rf, dmul(tlo, cf)), zhi = dadd(rf, dmul(thi, cf));
    const double lim = dadd((double)Re.cut, (double)1e-6f);
    const double dsnk = dsub((double)Re.L[f], zhi);
    if (dsub(dsnk, A.a) < lim) {
        fsnk[i] = 1;
        esnk[2 * i] = dsnk;
        esnk[2 * i + 1] = thi;
        atomicAdd(&cnt[2 * r], 1u);
    }
    if (dsub(zlo, A.a) < lim) {
        fsrc[i] = 1;
        esrc[2 * i] = zlo;
        esrc[2 * i + 1] = tlo;
        atomicAdd(&cnt[2 * r + 1], 1u);
    }
}

// Final contact arrays, per realisation block [internal | sink | source].
__global__ void k_final_internal(int R, const uint32_t* __restrict__ rodoff, uint32_t nrec,
                                 const Rec* __restrict__ rec, const uint32_t* __restrict__ keepf,
                                 const uint32_t* __restrict__ kscan, const uint32_t* __restrict__ rpos,
                                 const unsigned long long* __restrict__ ctoff, const Real* __restrict__ reals,
                                 const float4* __restrict__ pos, const float4* __restrict__ dir,
                                 uint32_t* __restrict__ oI, uint32_t* __restrict__ oJ, double* __restrict__ ot0,
                                 double* __restrict__ ot1, double* __restrict__ oD, double* __restrict__ oG,
                                 double* __restrict__ oS, int8_t* __restrict__ oimg, uint32_t* __restrict__ oreal) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrec || !keepf[q]) return;
    const Rec x = rec[q];
    int r = find_real(rodoff, R, x.i);
    const Real& Re = reals[r];
    uint32_t first = rpos[rodoff[r]];
    unsigned long long dst = ctoff[r] + (kscan[q] - kscan[first]);
    const RodD A = rodd(pos[x.i], dir[x.i]);
    const RodD B = rodd(pos[x.j], dir[x.j]);
    oI[dst] = x.i;
    oJ[dst] = x.j;
    ot0[dst] = x.t0;
    ot1[dst] = x.t1;
    oD[dst] = x.d;
    oG[dst] = tunnel_g(Re, dsub(dsub(x.d, A.a), B.a));
    const double sh[3] = {x.img[0] * (double)Re.L[0], x.img[1] * (double)Re.L[1], x.img[2] * (double)Re.L[2]};
    oS[dst] = contact_area(A, B, sh, x.Dx, x.u0, x.u1, (double)Re.cut);
    oimg[3 * dst + 0] = x.img[0];
    oimg[3 * dst + 1] = x.img[1];
    oimg[3 * dst + 2] = x.img[2];
    oreal[dst] = (uint32_t)r;
}

__global__ void k_final_elec(uint32_t nslot, int R, const uint32_t* __restrict__ rodoff,
                             const uint32_t* __restrict__ flag, const uint32_t* __restrict__ fscan,
                             const double* __restrict__ e, const unsigned long long* __restrict__ base,
                             uint32_t elec_id, const Real* __restrict__ reals, const float4* __restrict__ dir,
                             uint32_t* __restrict__ oI, uint32_t* __restrict__ oJ, double* __restrict__ ot0,
                             double* __restrict__ ot1, double* __restrict__ oD, double* __restrict__ oG,
                             double* __restrict__ oS, int8_t* __restrict__ oimg, uint32_t* __restrict__ oreal) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot || !flag[i]) return;
    int r = find_real(rodoff, R, i);
    const Real& Re = reals[r];
    unsigned long long dst = base[r] + (fscan[i] - fscan[rodoff[r]]);
    double D = e[2 * i];
    oI[dst] = i;
    oJ[dst] = elec_id;
    ot0[dst] = e[2 * i + 1];
    ot1[dst] = 0.0;
    oD[dst] = D;
    oG[dst] = tunnel_g(Re, dsub(D, (double)dir[i].w));
    oS[dst] = 0.0;
    oimg[3 * dst] = oimg[3 * dst + 1] = oimg[3 * dst + 2] = 0;
    oreal[dst] = (uint32_t)r;
}

// ---------------------------------------------------------------------------
#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

// Virtual rods of the screening as objects of the tube registration: the
// FP32 copy at the unwrapped centre; zero-length segments take no part.
struct TubeVirtSrc {
    const uint32_t* vcell;
    const Rec* rec;
    const uint32_t* rodoff;
    int R;
    const float4* vpf;
    const float4* vdf;
    __device__ bool operator()(uint32_t i, int* r, float4* p, float4* c) const {
        if (vcell[i] == 0xffffffffu) return false;
        *r = find_real(rodoff, R, rec[i].i);
        *p = vpf[i];
        *c = vdf[i];
        return true;
    }
    __device__ void geom(uint32_t i, float4* p, float4* c) const {
        *p = vpf[i];
        *c = vdf[i];
    }
};

nf_status Engine::contacts() {
    if (!cells_valid || rod_slots == 0) { err = "no rods: generate or set rods first"; return NF_ERR_STATE; }
    cudaEvent_t e0, e1;
    NF_CK(cudaEventCreate(&e0));
    NF_CK(cudaEventCreate(&e1));
    NF_CK(cudaEventRecord(e0, st));
    const uint64_t nrods = total_rods();
    const uint32_t nslot = (uint32_t)rod_slots;
    // Sorted rods: the cell list covers exactly the valid rods.
    NF_CK(cudaMemsetAsync(ctr.p + C_CT_PAIRS, 0, sizeof(unsigned long long) * (C_NCTR - C_CT_PAIRS), st));
    NF_CK(rcnt.ensure(nslot + 1));
    NF_CK(rpos.ensure(nslot + 1));
    NF_CK(rcur.ensure(nslot + 1));
    NF_CK(recn.ensure(2 * R + 2));
    size_t cap = std::max<size_t>(rec.cap, std::max<size_t>(4096, 2 * nrods));
    nf_status s = NF_OK;
    const unsigned xg = (unsigned)(4 * nsm);
    bool items_ok = false, done = false;
    for (int attempt = 0; attempt < 5 && !done; ++attempt) {
        if (!items_ok) {
            NF_CK(cudaMemsetAsync(ctr.p + C_ITEMS, 0, sizeof(unsigned long long), st));
            if (tube) {
                if (trod_stage != 1) {
                    s = tube_register_rods(1);
                    if (s != NF_OK) return s;
                    trod_stage = 1;
                }
                s = tube_items(trod_start.p, trod_start.p, nullptr, nullptr, true);
            } else {
                s = build_items(rstart.p, rstart.p, 1, nrods, nrods);
            }
            if (s != NF_OK) return s;
        }
        NF_CK(rec.ensure(cap));
        NF_CK(xq.ensure(xq_cap));
        if (tube) NF_CK(xqc.ensure(xq.cap));
        NF_CK(cudaMemsetAsync(rcnt.p, 0, sizeof(uint32_t) * (nslot + 1), st));
        NF_CK(cudaMemsetAsync(recn.p, 0, sizeof(unsigned long long), st));
        NF_CK(cudaMemsetAsync(ctr.p + C_XQ, 0, sizeof(unsigned long long), st));
        tstart(KT_CTPAIRS);
        if (nrods && tube) {
            NF_LAUNCH(k_tube_ct, persistent_grid(k_tube_ct), kTPB, 0, st)(dreal.p, R, toffs.p, titem_count(),
                                                   (uint32_t)titems.cap, titems.p, trod_start.p, trod_ent.p,
                                                   trod_pos.p, trod_dir.p,
                                                   xq.p, xqc.p, xq.cap, ctr.p);
            NF_CK(cudaGetLastError());
            NF_LAUNCH(k_ct_exact_tube, xg, 256, 0, st)(dreal.p, R, rodoff.p, xq.p, xqc.p, ctr.p + C_XQ, xq.cap,
                                                       pos.p, dir.p, rec.p, rec.cap, recn.p, rcnt.p, ctr.p);
        } else if (nrods) {
            NF_LAUNCH(k_ct_tiles, persistent_grid(k_ct_tiles), kTPB, 0, st)(dreal.p, item_count(), (uint32_t)items.cap, items.p, spos.p, sdir.p,
                                                   sid.p, xq.p, xq.cap, ctr.p);
            NF_CK(cudaGetLastError());
            NF_LAUNCH(k_ct_exact, xg, 256, 0, st)(dreal.p, R, rodoff.p, xq.p, ctr.p + C_XQ, xq.cap, spos.p, sdir.p,
                                                  sid.p, rec.p, rec.cap, recn.p, rcnt.p, ctr.p);
        }
        NF_CK(cudaGetLastError());
        tstop(KT_CTPAIRS);
        unsigned long long hv[4] = {0, 0, 0, 0};
        NF_CK(cudaMemcpyAsync(&hv[0], recn.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(&hv[1], ctr.p + C_XQ, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(&hv[2], ctr.p + C_ITEMS, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaMemcpyAsync(&hv[3], ctr.p + C_TUBE_OVF, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        if (hv[3]) { err = "tube registration beyond its bound"; return NF_ERR_OVERFLOW; }
        if (!tube && hv[2] > items.cap) { it_cap = (size_t)(hv[2] * 1.25) + 4096; items_ok = false; continue; }
        if (tube && hv[2] > titems.cap) { tit_cap = (size_t)(hv[2] * 1.25) + 4096; items_ok = false; continue; }
        items_ok = true;
        if (hv[1] > xq.cap) { xq_cap = (size_t)(hv[1] * 1.25) + 1024; continue; }
        if (hv[0] <= rec.cap) { cap = hv[0]; tbytes(KT_CTPAIRS, 36.0 * nrods + 64.0 * hv[0], 0); done = true; }
        else cap = hv[0] + hv[0] / 8 + 64;
    }
    if (!done) { err = "contact work list, queue or record buffer overflow"; return NF_ERR_OVERFLOW; }
    const uint32_t nrec = (uint32_t)cap;
    NF_CK(rec2.ensure(nrec + 1));
    s = scan_u32(rcnt.p, rpos.p, nslot + 1);
    if (s != NF_OK) return s;
    NF_CK(cudaMemsetAsync(rcur.p, 0, sizeof(uint32_t) * (nslot + 1), st));
    if (nrec) {
        NF_LAUNCH(k_rec_scatter, grid_for(nrec, 256), 256, 0, st)(nrec, rec.p, rpos.p, rcur.p, rec2.p);
        NF_CK(cudaGetLastError());
        NF_LAUNCH(k_rec_sort, grid_for(nslot, 256), 256, 0, st)(nslot, rpos.p, rcnt.p, rec2.p);
        NF_CK(cudaGetLastError());
        if (prm[0].screening) {
            NF_CK(vdbl.ensure((size_t)kVD * nrec));
            NF_CK(vpf.ensure(nrec));
            NF_CK(vdf.ensure(nrec));
            NF_CK(vcell.ensure(nrec));
            NF_CK(vperm.ensure(nrec));
            NF_CK(vstart.ensure(ncell + 1));
            NF_CK(vcur.ensure(ncell + 1));
            NF_CK(cudaMemsetAsync(vcur.p, 0, sizeof(uint32_t) * (ncell + 1), st));
            tstart(KT_SCREEN);
            NF_LAUNCH(k_virt, grid_for(nrec, 256), 256, 0, st)(R, rodoff.p, nrec, rec2.p, pos.p, dir.p, dreal.p, vdbl.p,
                                                               vpf.p, vdf.p, vcell.p, vcur.p);
            NF_CK(cudaGetLastError());
            s = scan_u32(vcur.p, vstart.p, ncell + 1);
            if (s != NF_OK) return s;
            NF_CK(cudaMemsetAsync(vcur.p, 0, sizeof(uint32_t) * (ncell + 1), st));
            NF_LAUNCH(k_vbin, grid_for(nrec, 256), 256, 0, st)(nrec, vcell.p, vstart.p, vcur.p, vperm.p);
            NF_CK(cudaGetLastError());
            bool vitems_ok = false, vdone = false;
            if (tube) {  // virtual rods on the tube grid, against the rods' stage-1 registrations
                TubeVirtSrc vsrc{vcell.p, rec2.p, rodoff.p, R, vpf.p, vdf.p};
                s = tube_register_objects(nrec, vsrc);
                if (s != NF_OK) return s;
            }
            for (int attempt = 0; attempt < 4 && !vdone; ++attempt) {
                if (!vitems_ok) {
                    NF_CK(cudaMemsetAsync(ctr.p + C_ITEMS, 0, sizeof(unsigned long long), st));
                    s = tube ? tube_items(tcnd_start.p, trod_start.p) : build_items(vstart.p, rstart.p, 1, nrec, nrods);
                    if (s != NF_OK) return s;
                }
                NF_CK(xq.ensure(xq_cap));
                NF_CK(cudaMemsetAsync(ctr.p + C_XQ, 0, sizeof(unsigned long long), st));
                if (tube) {
                    NF_LAUNCH(k_tube_scr, persistent_grid(k_tube_scr), kTPB, 0, st)(dreal.p, R, toffs.p, titem_count(),
                                                        (uint32_t)titems.cap, titems.p, tcnd_ent.p, tcnd_pos.p,
                                                        tcnd_dir.p, trod_ent.p, trod_pos.p, trod_dir.p, xq.p, xq.cap,
                                                        ctr.p);
                    NF_CK(cudaGetLastError());
                    NF_LAUNCH(k_scr_exact_tube, xg, 256, 0, st)(dreal.p, R, rodoff.p, xq.p, ctr.p + C_XQ, xq.cap,
                                                                vdbl.p, pos.p, dir.p, rec2.p, ctr.p);
                } else {
                    NF_LAUNCH(k_scr_tiles, persistent_grid(k_scr_tiles), kTPB, 0, st)(dreal.p, item_count(), (uint32_t)items.cap, items.p, vperm.p, vdbl.p,
                                                            vpf.p, vdf.p, spos.p, sdir.p, xq.p, xq.cap, ctr.p);
                    NF_CK(cudaGetLastError());
                    NF_LAUNCH(k_scr_exact, xg, 256, 0, st)(dreal.p, R, rodoff.p, xq.p, ctr.p + C_XQ, xq.cap, vdbl.p,
                                                           spos.p, sdir.p, rec2.p, ctr.p);
                }
                NF_CK(cudaGetLastError());
                unsigned long long nq[3] = {0, 0, 0};
                NF_CK(cudaMemcpyAsync(&nq[0], ctr.p + C_XQ, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
                NF_CK(cudaMemcpyAsync(&nq[1], ctr.p + C_ITEMS, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                      st));
                NF_CK(cudaMemcpyAsync(&nq[2], ctr.p + C_TUBE_OVF, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                      st));
                NF_CK(cudaStreamSynchronize(st));
                if (nq[2]) { err = "tube registration beyond its bound"; return NF_ERR_OVERFLOW; }
                // Screening flags are idempotent: an incomplete pass is simply rerun.
                if (tube && nq[1] > titems.cap) { tit_cap = (size_t)(nq[1] * 1.25) + 4096; vitems_ok = false; }
                else if (!tube && nq[1] > items.cap) { it_cap = (size_t)(nq[1] * 1.25) + 4096; vitems_ok = false; }
                else if (nq[0] > xq.cap) { vitems_ok = true; xq_cap = (size_t)(nq[0] * 1.25) + 1024; }
                else vdone = true;
            }
            if (!vdone) { err = "screening work list or queue overflow"; return NF_ERR_OVERFLOW; }
            tstop(KT_SCREEN);
            tbytes(KT_SCREEN, 64.0 * nrec + 32.0 * nrods, 0);
        }
    }
    // Counts per realisation.
    NF_CK(u32tmp.ensure(4 * (size_t)R + 2 * (size_t)nrec + 4 * (size_t)nslot + 16));
    uint32_t* cnt = u32tmp.p;                 // 4R: int, scr, snk, src
    uint32_t* keepf = cnt + 4 * R;            // nrec + 1
    uint32_t* kscan = keepf + nrec + 1;       // nrec + 1
    uint32_t* fsnk = kscan + nrec + 1;        // nslot + 1
    uint32_t* fsrc = fsnk + nslot + 1;
    uint32_t* ssnk = fsrc + nslot + 1;
    uint32_t* ssrc = ssnk + nslot + 1;
    // buffer-layer electrodes: the field axis of realisation 0 (every
    // realisation of a handle shares the electrode model and the field axis)
    const int faxis = hreal[0].ebuf ? hreal[0].field_axis : -1;
    DBuf<uint32_t>& xflag = ivals;  // reuse the intra-rod network's scratch
    DBuf<uint32_t>& xpos = ivals2;
    if (faxis >= 0) {
        NF_CK(xflag.ensure(nrec + 1));
        NF_CK(xpos.ensure(nrec + 1));
        NF_CK(cudaMemsetAsync(xflag.p, 0, sizeof(uint32_t) * (nrec + 1), st));
    }
    NF_CK(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * 4 * R, st));
    NF_CK(cudaMemsetAsync(keepf, 0, sizeof(uint32_t) * (nrec + 1), st));
    if (nrec) {
        NF_LAUNCH(k_rec_count, grid_for(nrec, 256), 256, 0, st)(R, rodoff.p, nrec, rec2.p, faxis, keepf,
                                                                 faxis >= 0 ? xflag.p : nullptr, cnt);
        NF_CK(cudaGetLastError());
    }
    s = scan_u32(keepf, kscan, nrec + 1);
    if (s != NF_OK) return s;
    if (faxis >= 0) {
        s = scan_u32(xflag.p, xpos.p, nrec + 1);
        if (s != NF_OK) return s;
    }
    DBuf<double>& esnk = vsnk;  // reuse solve buffers as scratch (2 doubles per slot)
    DBuf<double>& esrc = vsrc;
    NF_CK(esnk.ensure(2 * (size_t)nslot + 2));
    NF_CK(esrc.ensure(2 * (size_t)nslot + 2));
    NF_CK(cudaMemsetAsync(fsnk + nslot, 0, sizeof(uint32_t), st));
    NF_CK(cudaMemsetAsync(fsrc + nslot, 0, sizeof(uint32_t), st));
    if (faxis < 0) {  // plane electrodes
        NF_LAUNCH(k_elec, grid_for(nslot, 256), 256, 0, st)(nslot, R, rodoff.p, dcount.p, dreal.p, pos.p, dir.p, fsnk,
                                                            fsrc, esnk.p, esrc.p, cnt + 2 * R);
        NF_CK(cudaGetLastError());
        s = scan_u32(fsnk, ssnk, nslot + 1);
        if (s != NF_OK) return s;
        s = scan_u32(fsrc, ssrc, nslot + 1);
        if (s != NF_OK) return s;
    }
    std::vector<uint32_t> hc(4 * R);
    NF_CK(cudaMemcpyAsync(hc.data(), cnt, sizeof(uint32_t) * 4 * R, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    ct_int.assign(R, 0); ct_scr.assign(R, 0); ct_snk.assign(R, 0); ct_src.assign(R, 0);
    ct_off.assign(R + 1, 0);
    std::vector<unsigned long long> hoff(3 * R);
    for (int r = 0; r < R; ++r) {
        ct_int[r] = hc[2 * r]; ct_scr[r] = hc[2 * r + 1];
        ct_snk[r] = hc[2 * R + 2 * r]; ct_src[r] = hc[2 * R + 2 * r + 1];
        hoff[r] = ct_off[r];
        hoff[R + r] = ct_off[r] + ct_int[r];
        hoff[2 * R + r] = ct_off[r] + ct_int[r] + ct_snk[r];
        ct_off[r + 1] = ct_off[r] + ct_int[r] + ct_snk[r] + ct_src[r];
    }
    const size_t ntot = ct_off[R];
    NF_CK(cI.ensure(ntot + 1)); NF_CK(cJ.ensure(ntot + 1));
    NF_CK(ct0.ensure(ntot + 1)); NF_CK(ct1.ensure(ntot + 1));
    NF_CK(cD.ensure(ntot + 1)); NF_CK(cG.ensure(ntot + 1)); NF_CK(cS.ensure(ntot + 1));
    NF_CK(cimg.ensure(3 * ntot + 3)); NF_CK(creal2.ensure(ntot + 1));
    NF_CK(recn.ensure(3 * (size_t)R + 2));
    unsigned long long* doff = recn.p;
    NF_CK(cudaMemcpyAsync(doff, hoff.data(), sizeof(unsigned long long) * 3 * R, cudaMemcpyHostToDevice, st));
    if (nrec) {
        NF_LAUNCH(k_final_internal, grid_for(nrec, 256), 256, 0, st)(R, rodoff.p, nrec, rec2.p, keepf, kscan, rpos.p, doff,
                                                             dreal.p, pos.p, dir.p, cI.p, cJ.p, ct0.p, ct1.p, cD.p,
                                                             cG.p, cS.p, cimg.p, creal2.p);
        NF_CK(cudaGetLastError());
    }
    if (faxis < 0) {
        NF_LAUNCH(k_final_elec, grid_for(nslot, 256), 256, 0, st)(nslot, R, rodoff.p, fsnk, ssnk, esnk.p, doff + R,
                                                                  NF_SNK_ELEC, dreal.p, dir.p, cI.p, cJ.p, ct0.p,
                                                                  ct1.p, cD.p, cG.p, cS.p, cimg.p, creal2.p);
        NF_CK(cudaGetLastError());
        NF_LAUNCH(k_final_elec, grid_for(nslot, 256), 256, 0, st)(nslot, R, rodoff.p, fsrc, ssrc, esrc.p, doff + 2 * R,
                                                                  NF_SRC_ELEC, dreal.p, dir.p, cI.p, cJ.p, ct0.p,
                                                                  ct1.p, cD.p, cG.p, cS.p, cimg.p, creal2.p);
        NF_CK(cudaGetLastError());
    } else {
        // buffer layers: one sink and one source contact per cross record,
        // each list sorted by (rod, partner), ties in record order (stable)
        uint32_t nx = 0;
        std::vector<uint32_t> start(R + 1, 0);
        for (int r = 0; r < R; ++r) { start[r] = nx; nx += ct_snk[r]; }
        start[R] = nx;
        if (nx) {
            NF_CK(ikeys.ensure(2ull * nx));
            NF_CK(ikeys2.ensure(2ull * nx));
            NF_CK(inew.ensure(2ull * nx));
            NF_CK(igid.ensure(2ull * nx));
            NF_LAUNCH(k_buf_emit, grid_for(nrec, 256), 256, 0, st)(nrec, rec2.p, xflag.p, xpos.p, faxis, nx, ikeys.p,
                                                                  inew.p);
            NF_CK(cudaGetLastError());
            for (int h = 0; h < 2; ++h) {
                size_t bytes = 0;
                NF_CK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, ikeys.p + h * nx, ikeys2.p + h * nx,
                                                      inew.p + h * nx, igid.p + h * nx, (int)nx, 0, 64, st));
                NF_CK(cubtmp.ensure(bytes));
                NF_CK(cub::DeviceRadixSort::SortPairs(cubtmp.p, bytes, ikeys.p + h * nx, ikeys2.p + h * nx,
                                                      inew.p + h * nx, igid.p + h * nx, (int)nx, 0, 64, st));
                g_launches += 1;
            }
            DBuf<uint32_t>& dstart = rcur;  // free again: the record scatter is done
            NF_CK(dstart.ensure(R + 1));
            NF_CK(cudaMemcpyAsync(dstart.p, start.data(), sizeof(uint32_t) * (R + 1), cudaMemcpyHostToDevice, st));
            for (int h = 0; h < 2; ++h) {
                NF_LAUNCH(k_final_buf, grid_for(nx, 256), 256, 0, st)(
                    nx, ikeys2.p + h * nx, igid.p + h * nx, rec2.p, R, rodoff.p, dstart.p, doff + (h ? 2 * R : R),
                    h ? NF_SRC_ELEC : NF_SNK_ELEC, dreal.p, pos.p, dir.p, cI.p, cJ.p, ct0.p, ct1.p, cD.p, cG.p, cS.p,
                    cimg.p, creal2.p);
                NF_CK(cudaGetLastError());
            }
            NF_CK(cudaStreamSynchronize(st));  // the host start[] copy is in flight until here
        }
    }
    NF_CK(cudaEventRecord(e1, st));
    NF_CK(cudaEventSynchronize(e1));
    float ms = 0;
    NF_CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    unsigned long long hk[C_NCTR];
    NF_CK(cudaMemcpy(hk, ctr.p, sizeof(hk), cudaMemcpyDeviceToHost));
    std::memset(&cst, 0, sizeof(cst));
    for (int r = 0; r < R; ++r) {
        cst.contacts += ct_int[r];
        cst.screened += ct_scr[r];
        cst.n_sink += ct_snk[r];
        cst.n_source += ct_src[r];
    }
    cst.pair_tests = hk[C_CT_PAIRS] + hk[C_SCR_PAIRS];
    cst.exact_evals = hk[C_CT_EXACT] + hk[C_SCR_EXACT];
    cst.fp32_would_flip = hk[C_CT_FLIPS];
    cst.ms = ms;
    contacts_valid = true;
    contacts_screened = prm[0].screening != 0;
    solve_valid = false;
    int_valid = false;
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
