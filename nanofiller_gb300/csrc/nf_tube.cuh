// nf_tube.cuh -- the tube grid of the pair sweeps.
//
// Two rods whose reference distance is below a threshold thr have points P_A,
// P_B on their axis segments (extended to |t| <= l/2 + a + eps, where the
// reference routine takes its points) with |P_A - P_B| < thr; the midpoint of
// P_A and P_B lies within thr/2 of both segments. So if every object is
// registered in each cell of a grid that its segment, dilated by
// trho >= thr_max / 2, touches, every pair within reach shares a cell, and
// testing the pairs registered together in each cell finds all of them. For
// rods of length l in cells of edge e ~ l/4 an object registers in about
// 2 l / e + 1 cells holding ~64 registrations each (TUBE_LOAD), so a probe meets a few
// hundred targets instead of the ~4 000 of a 5 x 5 x 5 stencil of cells of
// edge reach / 2 at 2 % volume fraction.
//
// A pair can share several cells, so it can be tested more than once. The
// boolean tests (a candidate against placed rods, screening) do not mind. A
// record (a contact, an in-round conflict) is written only by the cell that
// holds the midpoint of the pair's two points (tube_claims, tube_claims_d):
// the points of a pair within reach are closer than the threshold, so their
// midpoint lies within trho of both segments and its cell holds both
// objects. FP64-decided conflicts may be listed twice; the in-order
// resolution reads a list as a set.
//
// Registration entry: object id << 6 | image code, the image (x, y, z in
// -1..1, 2 bits each, +1) of the object's copy that the cell holds (on a
// periodic axis an object near a face also registers in the cells across
// it). Open axes have margin cells beyond both faces instead.
#pragma once
#include <cstdint>

#include "nf_common.cuh"
#include "nf_tiles.cuh"

#include <cooperative_groups.h>
#include <algorithm>
#include <cmath>

namespace nf {

constexpr uint32_t kTubeIdShift = 6;
// An entry slot left free in a cell (image code 3 on every axis: no entry).
constexpr uint32_t kTubeRoom = 0xffffffffu;

__host__ __device__ __forceinline__ uint32_t tube_entry(uint32_t id, const int img[3]) {
    return (id << kTubeIdShift) | (uint32_t)(img[0] + 1) | ((uint32_t)(img[1] + 1) << 2) |
           ((uint32_t)(img[2] + 1) << 4);
}

__host__ __device__ __forceinline__ void tube_unpack(uint32_t e, uint32_t* id, int img[3]) {
    *id = e >> kTubeIdShift;
    img[0] = (int)(e & 3u) - 1;
    img[1] = (int)((e >> 2) & 3u) - 1;
    img[2] = (int)((e >> 4) & 3u) - 1;
}

// Wraps unwrapped cell index u[3] for the stage's periodic mask: the global
// cell and the image of the object's copy in it; false when the cell lies
// beyond the margin of an open axis.
__device__ __forceinline__ bool tube_cell(const Real& R, int per, const int u[3], uint32_t* cell, int img[3]) {
    int w[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int n = R.tcn[d];
        int v = u[d], im = 0;
        if ((per >> d) & 1) {
            if (v < 0) { v += n; im = 1; }         // the copy shifted by +L lands here
            else if (v >= n) { v -= n; im = -1; }  // the copy shifted by -L
            if (v < 0 || v >= n) return false;     // beyond one image (excluded by set-up)
        } else {
            v += R.tcm[d];
            if (v < 0 || v >= n + 2 * R.tcm[d]) return false;
        }
        w[d] = v;
        img[d] = im;
    }
    const uint32_t nx = (uint32_t)(R.tcn[0] + 2 * R.tcm[0]), ny = (uint32_t)(R.tcn[1] + 2 * R.tcm[1]);
    *cell = R.toff + (uint32_t)w[0] + nx * ((uint32_t)w[1] + ny * (uint32_t)w[2]);
    return true;
}

// Visits every cell (global id, image of the copy) that the object's axis
// segment, extended to h = (l/2 + a + eps) and dilated by trho, touches:
// slabs of cells along the axis's dominant direction, in each the cells of the
// bounding box of the slab's piece of segment (the slab widened by trho),
// widened by trho. Every point within trho of the segment is inside a
// visited cell; no cell is visited twice. FP32 throughout; trho carries
// margins far above its rounding.
template <class F>
__device__ __forceinline__ void tube_walk(const Real& R, int per, const float4& p, const float4& c, F&& visit) {
    const float h = (p.w * 0.5f + c.w + R.eps) * 1.00001f + R.slack;
    const float rho = R.trho;
    const float pc[3] = {p.x, p.y, p.z}, cc[3] = {c.x, c.y, c.z};
    const float ax = fabsf(c.x), ay = fabsf(c.y), az = fabsf(c.z);
    const int d = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
    const int o1 = d == 0 ? 1 : 0, o2 = d == 2 ? 1 : 2;
    const float e0 = pc[d] - h * cc[d], e1 = pc[d] + h * cc[d];
    const float lo = fminf(e0, e1) - rho, hi = fmaxf(e0, e1) + rho;
    const int s0 = (int)floorf(lo * R.tci[d]), s1 = (int)floorf(hi * R.tci[d]);
    const float inv_cd = 1.0f / cc[d];
    for (int s = s0; s <= s1; ++s) {
        const float x0 = (float)s * R.tce[d] - rho, x1 = (float)(s + 1) * R.tce[d] + rho;
        const float ta = (x0 - pc[d]) * inv_cd, tb = (x1 - pc[d]) * inv_cd;
        const float t0 = fmaxf(fminf(ta, tb), -h), t1 = fminf(fmaxf(ta, tb), h);
        if (t0 > t1) continue;
        const float qa1 = pc[o1] + t0 * cc[o1], qb1 = pc[o1] + t1 * cc[o1];
        const float qa2 = pc[o2] + t0 * cc[o2], qb2 = pc[o2] + t1 * cc[o2];
        const int y0 = (int)floorf((fminf(qa1, qb1) - rho) * R.tci[o1]);
        const int y1 = (int)floorf((fmaxf(qa1, qb1) + rho) * R.tci[o1]);
        const int z0 = (int)floorf((fminf(qa2, qb2) - rho) * R.tci[o2]);
        const int z1 = (int)floorf((fmaxf(qa2, qb2) + rho) * R.tci[o2]);
        for (int y = y0; y <= y1; ++y)
            for (int z = z0; z <= z1; ++z) {
                int u[3];
                u[d] = s;
                u[o1] = y;
                u[o2] = z;
                uint32_t cell;
                int img[3];
                if (tube_cell(R, per, u, &cell, img)) visit(cell, img);
            }
    }
}

// Warp-private staging of one tile of target entries.
struct TubeTile {
    float4 ps[kWT];  // target copy centre, .w = its reach term of the capsule test
    float4 p[kWT];   // target centre (original coordinates), .w = length
    float4 c[kWT];   // axis, .w = radius
    uint32_t id[kWT];
    uint32_t im[kWT];  // image code of the target's copy
};

__device__ __forceinline__ void img_of(uint32_t code, int img[3]) {
    img[0] = (int)(code & 3u) - 1;
    img[1] = (int)((code >> 2) & 3u) - 1;
    img[2] = (int)((code >> 4) & 3u) - 1;
}

// Relative image of a pair (target copy image - probe copy image); false when
// it is beyond one box (such a pair is farther apart than a box edge).
__device__ __forceinline__ bool rel_img(uint32_t ip, uint32_t it, int img[3]) {
    int a[3], b[3];
    img_of(ip, a);
    img_of(it, b);
    bool ok = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        img[d] = b[d] - a[d];
        ok = ok && img[d] >= -1 && img[d] <= 1;
    }
    return ok;
}

// Whether the tube cell `cell`, holding the probe's copy of image code ip,
// is the one cell that claims a pair whose points are P_A = A + t0 cA and
// P_B = B + img L + t1 cB: the cell of their midpoint in A's frame (both
// objects are registered there: the midpoint is within the pair's distance /
// 2 of both segments).
__device__ __forceinline__ bool tube_claims(const Real& Re, int per, uint32_t cell, uint32_t ip, const float4& pA,
                                            const float4& cA, const float4& pB, const float4& cB, float sx, float sy,
                                            float sz, float t0, float t1) {
    const float mx = 0.5f * ((pA.x + t0 * cA.x) + ((pB.x + sx) + t1 * cB.x));
    const float my = 0.5f * ((pA.y + t0 * cA.y) + ((pB.y + sy) + t1 * cB.y));
    const float mz = 0.5f * ((pA.z + t0 * cA.z) + ((pB.z + sz) + t1 * cB.z));
    const int u[3] = {(int)floorf(mx * Re.tci[0]), (int)floorf(my * Re.tci[1]), (int)floorf(mz * Re.tci[2])};
    uint32_t c2;
    int im[3];
    if (!tube_cell(Re, per, u, &c2, im)) return false;
    return c2 == cell && tube_entry(0, im) == (ip & 63u);
}

// Exact-queue append that also records the tube cell the pair came from.
__device__ __forceinline__ void xq_push_cell(unsigned long long* q, uint32_t* qc, unsigned long long cap,
                                             unsigned long long* count, unsigned long long e, uint32_t cell) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (unsigned long long)g.size());
    base = g.shfl(base, 0);
    const unsigned long long slot = base + g.thread_rank();
    if (slot < cap) {
        q[slot] = e;
        qc[slot] = cell;
    }
}

// tube_claims in FP64 (the points of the FP64 routine): the cell of the
// midpoint of P_A = A + t0 cA and P_B = B + s + t1 cB in A's frame.
__device__ __forceinline__ bool tube_claims_d(const Real& Re, int per, uint32_t cell, const RodD& A, const RodD& B,
                                              double sx, double sy, double sz, double t0, double t1) {
    const double mx = dmul(0.5, dadd(dadd(A.x, dmul(t0, A.cx)), dadd(dadd(B.x, sx), dmul(t1, B.cx))));
    const double my = dmul(0.5, dadd(dadd(A.y, dmul(t0, A.cy)), dadd(dadd(B.y, sy), dmul(t1, B.cy))));
    const double mz = dmul(0.5, dadd(dadd(A.z, dmul(t0, A.cz)), dadd(dadd(B.z, sz), dmul(t1, B.cz))));
    const int u[3] = {(int)floor(mx * (double)Re.tci[0]), (int)floor(my * (double)Re.tci[1]),
                      (int)floor(mz * (double)Re.tci[2])};
    uint32_t c2;
    int im[3];
    return tube_cell(Re, per, u, &c2, im) && c2 == cell;
}

// Registration of a set of objects: count pass (per-cell totals) and fill
// pass (entries at start[cell] + cursor). Src(i, &real, &p, &c) gives object
// i's realisation and geometry, or false when it takes no part.
//
// One object per lane would leave most lanes idle (objects that take no part,
// segments with fewer slabs than their neighbours), so a warp first lists the
// slabs of its 32 objects (warp prefix sum of the slab counts) and then hands
// them out 32 at a time: lane g takes slab g of the list, finds its object by
// a binary search over the prefix and visits that slab's cells.
constexpr int kRegTPB = 256;

// kMode: 0 count pass, 1 fill pass, 2 append (objects added to a registration
// that left room in its cells: entry and geometry at start[cell] + the cell's
// count when below start[cell + 1], else the count is restored and the
// registration counted in ovf).
template <class Src, int kMode>
__global__ void __launch_bounds__(kRegTPB) k_treg(uint32_t n, const uint32_t* __restrict__ ntot,
                                                  const Real* __restrict__ reals, int stage, Src src,
                                                  uint32_t* __restrict__ tcnt, const uint32_t* __restrict__ tstart,
                                                  uint32_t* __restrict__ tent, float4* __restrict__ tpos,
                                                  float4* __restrict__ tdir, uint32_t cap,
                                                  unsigned long long* __restrict__ ovf) {
    constexpr int kW = kRegTPB / 32;
    __shared__ float4 sp[kW][32], sc[kW][32];
    __shared__ int sr[kW][32], ss0[kW][32], sex[kW][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lim = ntot ? *ntot : n;
    int r = 0;
    float4 p = make_float4(0, 0, 0, 0), c = p;
    int ns = 0, s0 = 0;
    if (i < lim && src(i, &r, &p, &c)) {
        const Real& Re = reals[r];
        const float h = (p.w * 0.5f + c.w + Re.eps) * 1.00001f + Re.slack;
        const float pc[3] = {p.x, p.y, p.z}, cc[3] = {c.x, c.y, c.z};
        const float ax = fabsf(c.x), ay = fabsf(c.y), az = fabsf(c.z);
        const int d = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
        const float e0 = pc[d] - h * cc[d], e1 = pc[d] + h * cc[d];
        s0 = (int)floorf((fminf(e0, e1) - Re.trho) * Re.tci[d]);
        const int s1 = (int)floorf((fmaxf(e0, e1) + Re.trho) * Re.tci[d]);
        ns = s1 - s0 + 1;
    }
    int incl = ns;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    sp[w][lane] = p;
    sc[w][lane] = c;
    sr[w][lane] = r;
    ss0[w][lane] = s0;
    sex[w][lane] = incl - ns;
    __syncwarp();
    for (int base = 0; base < total; base += 32) {
        const int g = base + lane;
        if (g >= total) break;
        int l = 0;
#pragma unroll
        for (int step = 16; step; step >>= 1)
            if (l + step < 32 && sex[w][l + step] <= g) l += step;
        const Real& Re = reals[sr[w][l]];
        const int per = stage ? Re.per_con : Re.per_gen;
        const float4 q = sp[w][l], cq = sc[w][l];
        const uint32_t id = i - (uint32_t)lane + (uint32_t)l;
        const int s = ss0[w][l] + (g - sex[w][l]);
        // the cells of slab s of object id (tube_walk's slab loop body)
        const float h = (q.w * 0.5f + cq.w + Re.eps) * 1.00001f + Re.slack;
        const float rho = Re.trho;
        const float pc[3] = {q.x, q.y, q.z}, cc[3] = {cq.x, cq.y, cq.z};
        const float ax = fabsf(cq.x), ay = fabsf(cq.y), az = fabsf(cq.z);
        const int d = (ax >= ay && ax >= az) ? 0 : (ay >= az ? 1 : 2);
        const int o1 = d == 0 ? 1 : 0, o2 = d == 2 ? 1 : 2;
        const float inv_cd = 1.0f / cc[d];
        const float x0 = (float)s * Re.tce[d] - rho, x1 = (float)(s + 1) * Re.tce[d] + rho;
        const float ta = (x0 - pc[d]) * inv_cd, tb = (x1 - pc[d]) * inv_cd;
        const float t0 = fmaxf(fminf(ta, tb), -h), t1 = fminf(fmaxf(ta, tb), h);
        if (t0 > t1) continue;
        const float qa1 = pc[o1] + t0 * cc[o1], qb1 = pc[o1] + t1 * cc[o1];
        const float qa2 = pc[o2] + t0 * cc[o2], qb2 = pc[o2] + t1 * cc[o2];
        const int y0 = (int)floorf((fminf(qa1, qb1) - rho) * Re.tci[o1]);
        const int y1 = (int)floorf((fmaxf(qa1, qb1) + rho) * Re.tci[o1]);
        const int z0 = (int)floorf((fminf(qa2, qb2) - rho) * Re.tci[o2]);
        const int z1 = (int)floorf((fmaxf(qa2, qb2) + rho) * Re.tci[o2]);
        for (int y = y0; y <= y1; ++y)
            for (int z = z0; z <= z1; ++z) {
                int u[3];
                u[d] = s;
                u[o1] = y;
                u[o2] = z;
                uint32_t cell;
                int img[3];
                if (!tube_cell(Re, per, u, &cell, img)) continue;
                if (kMode == 1) {
                    const uint32_t qd = tstart[cell] + atomicAdd(&tcnt[cell], 1u);
                    if (qd < cap) tent[qd] = tube_entry(id, img);
                    else atomicAdd(ovf, 1ull);
                } else if (kMode == 2) {
                    const uint32_t qd = tstart[cell] + atomicAdd(&tcnt[cell], 1u);
                    if (qd < tstart[cell + 1]) {
                        tent[qd] = tube_entry(id, img);
                        tpos[qd] = q;
                        tdir[qd] = cq;
                    } else {
                        // a count never ends above the room: every increment
                        // that found the cell full is taken back
                        atomicSub(&tcnt[cell], 1u);
                        atomicAdd(ovf, 1ull);
                    }
                } else {
                    atomicAdd(&tcnt[cell], 1u);
                }
            }
    }
}

// The objects' geometry beside their entries (the sweeps then read it
// coalesced): entry q's object through the source's geometry accessor, read
// at random, written in entry order.
template <class Src>
__global__ void __launch_bounds__(256) k_treg_geom(uint32_t n, const uint32_t* __restrict__ ent,
                                                   float4* __restrict__ epos, float4* __restrict__ edir, Src src) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const uint32_t e = ent[q];
        if (e == kTubeRoom) continue;  // room left in a cell for later objects
        float4 p, c;
        src.geom(e >> kTubeIdShift, &p, &c);
        epos[q] = p;
        edir[q] = c;
    }
}

// Room per cell for the objects later rounds add (a registration that is
// appended to): on entry cnt[c] holds the cell's count k, on exit its
// capacity (1 + g) (k + 3 sqrt(k + 1) + 3) + 8, g the growth expected for its
// realisation (objects to come over present ones): a Poisson count k puts
// the cell's final count below (1 + g) (k + 3 sqrt(k + 1) + 3) at about
// three standard deviations, so a cell runs out of room rarely even when k
// is a small sample of it.
static __global__ void k_treg_room(uint32_t ncell, uint32_t* __restrict__ cnt, const uint32_t* __restrict__ toffs,
                                   int R, const float* __restrict__ grow) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const float k = (float)cnt[c];
    const float g = grow[find_real(toffs, R, c)];
    cnt[c] = (uint32_t)ceilf((1.0f + g) * (k + 3.0f * sqrtf(k + 1.0f) + 3.0f)) + 8u;
}

// In-place compaction of a candidate registration to the candidates still
// alive (the survivors of the old-rod test), one warp per cell: the list of
// each cell keeps its order and its start; cnt[c] receives its new length.
// A chunk of 32 entries is read before any of it is written, and writes go to
// positions at or below the chunk's, so no entry is overwritten unread.
static __global__ void k_treg_compact(uint32_t ncell, const uint32_t* __restrict__ start, uint32_t* __restrict__ cnt,
                                      uint32_t* __restrict__ ent, float4* __restrict__ epos, float4* __restrict__ edir,
                                      const uint8_t* __restrict__ state, uint8_t alive_state) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const unsigned lt = (1u << lane) - 1u;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncell; c += nw) {
        const uint32_t b = start[c], e = start[c + 1];
        uint32_t w = b;
        for (uint32_t k = b; k < e; k += 32) {
            const uint32_t i = k + lane;
            const bool valid = i < e;
            uint32_t en = 0;
            float4 p = make_float4(0, 0, 0, 0), d = p;
            if (valid) { en = ent[i]; p = epos[i]; d = edir[i]; }
            const bool alive = valid && state[en >> kTubeIdShift] == alive_state;
            const unsigned bal = __ballot_sync(0xffffffffu, alive);
            __syncwarp();
            if (alive) {
                const uint32_t q = w + __popc(bal & lt);
                ent[q] = en;
                epos[q] = p;
                edir[q] = d;
            }
            w += __popc(bal);
            __syncwarp();
        }
        if (lane == 0) cnt[c] = w - b;
    }
}

// Work items of the tube sweeps. Item layout (16 B): first probe entry,
// first target entry, cell, count word.
// - A cell item: probe chunks of <= 32 times target segments of <= kTSeg of
//   one cell; count word np | nt << 6 | realisation << 14.
// - A packed item (kPackBit set): a run of consecutive cells from `cell`, of
//   one realisation (in the first word), whose small cells (1-32 probes and
//   1-32 targets each) hold <= 32 probes and <= 32 targets together; count
//   word span | np << 6 | nt << 12 | bit. A lane takes one probe of any of
//   them and tests it against its own cell's targets, so the warp's lanes
//   fill up where cells hold a few objects each.
// Cells that are not small get cell items. With more realisations than the
// count word holds (kItemRealMax), cell items carry none and the sweeps look
// it up.
constexpr uint32_t kTSeg = 128;
constexpr uint32_t kPackBit = 0x80000000u;
constexpr int kItemRealMax = (1 << 17) - 1;

// Realisation of item I (whose count word is cnt) for R realisations.
__device__ __forceinline__ int item_real(uint32_t pfirst, uint32_t cnt, uint32_t cell, const uint32_t* toffs, int R) {
    if (cnt & kPackBit) return (int)pfirst;
    if (R <= kItemRealMax) return (int)((cnt >> 14) & 0x1FFFFu);
    return find_real(toffs, R, cell);
}

// Entries of cell c: [start[c], start[c] + cnt[c]) when a count array is
// given (a list compacted in place), else [start[c], start[c + 1]).
__device__ __forceinline__ uint32_t tube_count(const uint32_t* start, const uint32_t* cnt, uint32_t c) {
    return cnt ? cnt[c] : start[c + 1] - start[c];
}

__device__ __forceinline__ bool tube_small(uint32_t np, uint32_t nt) {
    return np != 0u && nt != 0u && np <= 32u && nt <= 32u;
}

struct TItem {
    uint32_t pfirst, tfirst, cell, cnt;
};

__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, int lane, uint32_t* total) {
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    *total = __shfl_sync(0xffffffffu, incl, 31);
    return incl - v;
}

// One warp per segment of 32 consecutive cells: count pass (items per
// segment into icnt) or fill pass (items at ioff[segment]). With pack, the
// segment's small cells go into packed items, greedily in cell order; the
// other cells (and every cell without pack) get cell items.
template <bool kFill>
__global__ void __launch_bounds__(256) k_titem(uint32_t ncell, int pack, const uint32_t* __restrict__ toffs, int R,
                                               const uint32_t* __restrict__ pstart,
                                               const uint32_t* __restrict__ tstart, const uint32_t* __restrict__ pcnt,
                                               const uint32_t* __restrict__ tcnt, uint32_t* __restrict__ icnt,
                                               const uint32_t* __restrict__ ioff, TItem* __restrict__ items,
                                               uint32_t cap, unsigned long long* __restrict__ imax) {
    const int lane = threadIdx.x & 31;
    const uint32_t nseg = (ncell + 31u) / 32u;
    if (kFill && blockIdx.x == 0 && threadIdx.x == 0) atomicMax(imax, (unsigned long long)ioff[nseg]);
    if (!kFill && blockIdx.x == 0 && threadIdx.x == 0) icnt[nseg] = 0;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t sg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sg < nseg; sg += nw) {
        const uint32_t c = sg * 32u + (uint32_t)lane;
        uint32_t np = 0, nt = 0;
        if (c < ncell) {
            np = tube_count(pstart, pcnt, c);
            nt = tube_count(tstart, tcnt, c);
        }
        const bool small = pack && tube_small(np, nt);
        const uint32_t nbig = (!small && np && nt) ? ((np + 31u) / 32u) * ((nt + kTSeg - 1u) / kTSeg) : 0u;
        const int rl = (np && nt) ? find_real(toffs, R, min(c, ncell - 1u)) : 0;
        // greedy groups of the small cells: a group ends before the first
        // small cell that would take it past 32 probes or 32 targets, or that
        // belongs to another realisation
        uint32_t ta, tb;
        const uint32_t ea = warp_excl_scan(small ? np : 0u, lane, &ta);
        const uint32_t eb = warp_excl_scan(small ? nt : 0u, lane, &tb);
        const uint32_t ia = ea + (small ? np : 0u), ib = eb + (small ? nt : 0u);
        unsigned starts = 0;
        const unsigned smask = __ballot_sync(0xffffffffu, small);
        if (smask) {
            int g = __ffs(smask) - 1;
            for (;;) {
                starts |= 1u << g;
                const uint32_t ba = __shfl_sync(0xffffffffu, ea, g), bb = __shfl_sync(0xffffffffu, eb, g);
                const int rg = __shfl_sync(0xffffffffu, rl, g);
                const unsigned over =
                    __ballot_sync(0xffffffffu, lane > g && small && (ia - ba > 32u || ib - bb > 32u || rl != rg));
                if (!over) break;
                g = __ffs(over) - 1;
            }
        }
        const bool st = (starts >> lane) & 1u;
        uint32_t tot;
        const uint32_t off = warp_excl_scan((st ? 1u : 0u) + nbig, lane, &tot);
        // every lane's group end (the next start, or the segment's end)
        const unsigned later = starts & ~((2u << lane) - 1u);
        const int end = later ? __ffs(later) - 1 : 32;
        const uint32_t ia_end = __shfl_sync(0xffffffffu, ia, end - 1), ib_end = __shfl_sync(0xffffffffu, ib, end - 1);
        if (!kFill) {
            if (lane == 0) icnt[sg] = tot;
            continue;
        }
        uint32_t k = ioff[sg] + off;
        if (st && k < cap) {
            const uint32_t span = (uint32_t)(end - lane), gp = ia_end - ea, gt = ib_end - eb;
            items[k] = TItem{(uint32_t)rl, 0u, c, kPackBit | span | (gp << 6) | (gt << 12)};
        }
        k += st ? 1u : 0u;
        if (nbig) {
            const uint32_t p0 = pstart[c], t0 = tstart[c];
            const uint32_t segs = (nt + kTSeg - 1u) / kTSeg;
            for (uint32_t idx = 0; idx < nbig && k + idx < cap; ++idx) {
                const uint32_t a = (idx / segs) * 32u, b = (idx % segs) * kTSeg;
                const uint32_t pa = min(32u, np - a), tb2 = min(kTSeg, nt - b);
                const uint32_t rw = R <= kItemRealMax ? (uint32_t)rl << 14 : 0u;
                items[k + idx] = TItem{p0 + a, t0 + b, c, pa | (tb2 << 6) | rw};
            }
        }
    }
}

// The cells of a packed item, one per lane of the warp's scratch: prefix of
// probes and targets (P, Q; 0xffffffff past the span), first entries, counts.
struct TubePack {
    uint32_t P[32], Q[32], ps[32], ts[32], np[32], nt[32];
};

// Fills pk for packed item I (all lanes); returns nothing, counts from I.
__device__ __forceinline__ void tube_pack_load(const TItem& I, int lane, const uint32_t* __restrict__ pstart,
                                               const uint32_t* __restrict__ tstart, const uint32_t* __restrict__ pcnt,
                                               const uint32_t* __restrict__ tcnt, TubePack& pk) {
    const uint32_t span = I.cnt & 63u;
    uint32_t a = 0, b = 0, ps = 0, ts = 0;
    if ((uint32_t)lane < span) {
        const uint32_t c = I.cell + (uint32_t)lane;
        const uint32_t np = tube_count(pstart, pcnt, c), nt = tube_count(tstart, tcnt, c);
        if (tube_small(np, nt)) {
            a = np;
            b = nt;
            ps = pstart[c];
            ts = tstart[c];
        }
    }
    uint32_t ta, tb;
    const uint32_t ea = warp_excl_scan(a, lane, &ta), eb = warp_excl_scan(b, lane, &tb);
    __syncwarp();
    pk.P[lane] = (uint32_t)lane < span ? ea : 0xffffffffu;
    pk.Q[lane] = (uint32_t)lane < span ? eb : 0xffffffffu;
    pk.ps[lane] = ps;
    pk.ts[lane] = ts;
    pk.np[lane] = a;
    pk.nt[lane] = b;
    __syncwarp();
}

// The cell (lane of pk) holding slot j of prefix X: the last k with X[k] <= j.
__device__ __forceinline__ int tube_pack_find(const uint32_t* X, uint32_t j) {
    int k = 0;
#pragma unroll
    for (int step = 16; step; step >>= 1)
        if (X[k + step] <= j) k += step;
    return k;
}

// Probe side of item I for this lane: entry index, cell, and (packed items)
// the lane's target range in the tile; np / nt the item's probe and target
// counts.
struct TubeLane {
    uint32_t np, nt, pe, cell, tlo, tlen;
    bool packed;
};

__device__ __forceinline__ TubeLane tube_lane(const TItem& I, int lane, const uint32_t* __restrict__ pstart,
                                              const uint32_t* __restrict__ tstart, const uint32_t* __restrict__ pcnt,
                                              const uint32_t* __restrict__ tcnt, TubePack& pk) {
    TubeLane L;
    L.packed = (I.cnt & kPackBit) != 0u;
    L.cell = I.cell;
    L.tlo = 0;
    L.tlen = 0;
    if (L.packed) {
        tube_pack_load(I, lane, pstart, tstart, pcnt, tcnt, pk);
        L.np = (I.cnt >> 6) & 63u;
        L.nt = (I.cnt >> 12) & 63u;
        L.pe = 0;
        if ((uint32_t)lane < L.np) {
            const int k = tube_pack_find(pk.P, (uint32_t)lane);
            L.pe = pk.ps[k] + ((uint32_t)lane - pk.P[k]);
            L.cell = I.cell + (uint32_t)k;
            L.tlo = pk.Q[k];
            L.tlen = pk.nt[k];
        }
    } else {
        L.np = I.cnt & 63u;
        L.nt = (I.cnt >> 6) & 0xFFu;
        L.pe = I.pfirst + (uint32_t)lane;
    }
    return L;
}

// Target entry of tile slot `slot` (< the tile's count) of stage b, and its cell.
__device__ __forceinline__ uint32_t tube_target(const TItem& I, const TubeLane& L, const TubePack& pk, uint32_t b,
                                                uint32_t slot, uint32_t* cell) {
    if (L.packed) {
        const int k = tube_pack_find(pk.Q, slot);
        *cell = I.cell + (uint32_t)k;
        return pk.ts[k] + (slot - pk.Q[k]);
    }
    *cell = I.cell;
    return I.tfirst + b + slot;
}

}  // namespace nf
