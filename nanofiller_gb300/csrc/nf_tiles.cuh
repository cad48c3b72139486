// nf_tiles.cuh -- work decomposition of the cell-pair kernels.
//
// Probes (candidates, rods or virtual rods) and targets are binned by cell
// (CSR pstart / tstart). The pair kernels run over a work list built on the
// device: one item per (probe chunk of <= kWC = 32 probes of a cell, stencil
// offset, segment of <= kSeg targets of the neighbour cell), so no item is
// longer than kSeg targets whatever the density, and empty neighbours (open
// boundaries, empty cells) produce no items. A persistent grid of 4-warp
// blocks strides over the items; a warp takes one item, each lane holds one
// probe, the warp stages the segment's targets 32 at a time in its own
// shared-memory tile (one coalesced load per lane) and every lane tests its
// probe against each staged target (broadcast reads, no bank conflict).
// (The generation's tube-grid kernels mark pair-parallel instead: an item's
// live probes share the warp's lanes, 2^s lanes per probe, so that items of
// few probes keep every lane marking; in the contact sweep the same measured
// 4 % slower.) Warps only meet at __syncwarp.
#pragma once
#include <cstdint>

#include <cooperative_groups.h>

#include "nf_common.cuh"

namespace nf {

constexpr int kTPB = 128;   // threads per block of the pair kernels (4 independent warps)
constexpr int kWC = 32;     // probes per item: one per lane
constexpr int kWT = 32;     // targets per warp-private shared-memory tile
constexpr int kSeg = 128;   // targets per item at most

// Pairs that pass the per-lane capsule pre-test are marked in a 32-bit mask
// per lane (bit j = staged target j); after the tile the marked pairs are
// handed out 32 at a time to the whole warp, so the long filter path
// (maybe_near, certain_hit) runs with every lane busy. A far-away position
// pads the tile beyond its last target, so the marking loop needs no bound.
constexpr float kFar = 1.0e30f;

// Capsule pre-test of the marking loops (replaces a bounding-sphere test and
// implies it). The reference's distance is taken between points of the two
// axis segments extended to |t| <= h = l/2 + a + eps, so a pair with d < thr
// has its target's centre within hB|cB| + thr of the probe's extended segment.
// b = target centre - probe centre (image shift included), c = probe axis,
// h = probe extent, hBt = (hB + a_B-part of thr) * 1.000002 (staged with the
// target), hC = (probe part of thr) * 1.000002 + slack + 4e-6 (1 + probe
// reach). The 4e-6 relative terms cover FP32 rounding of the projection and of
// the squares and |c| = 1 +- 1e-6 (the same margins as maybe_near); slack
// covers the rounding of the coordinates. Far tile padding overflows r^2 to inf
// and fails the test.
__device__ __forceinline__ bool capsule_near(float bx, float by, float bz, float cx, float cy, float cz, float h,
                                             float hBt, float hC) {
    float t = bx * cx + by * cy + bz * cz;
    t = fminf(fmaxf(t, -h), h);
    const float rx = fmaf(-t, cx, bx), ry = fmaf(-t, cy, by), rz = fmaf(-t, cz, bz);
    const float R = fmaf(hBt, 1.000004f, hC);
    return rx * rx + ry * ry + rz * rz <= R * R;
}

// Position of the k-th (from 0) set bit of m, k < popc(m): a binary search on
// population counts of halves, quarters, ... (no loop, no divergence).
__device__ __forceinline__ int nth_set_bit(uint32_t m, int k) {
    int pos = 0, c = __popc(m & 0xffffu);
    if (k >= c) { k -= c; m >>= 16; pos = 16; }
    c = __popc(m & 0xffu);
    if (k >= c) { k -= c; m >>= 8; pos += 8; }
    c = __popc(m & 0xfu);
    if (k >= c) { k -= c; m >>= 4; pos += 4; }
    c = __popc(m & 0x3u);
    if (k >= c) { k -= c; m >>= 2; pos += 2; }
    return pos + (k >= (int)(m & 1u) ? 1 : 0);
}

// Hands the marked pairs of a tile to the warp in two stages. Stage 1: 32 at a
// time, keep(probe_lane, slot) runs a cheap rejection (one lane per pair).
// Stage 2: the pairs kept are gathered in a second per-warp list q2 (64 entries)
// and eval(valid, probe_lane, slot) runs on 32 of them at a time, so the long
// evaluation also runs with every lane busy. eval is called by all lanes
// (valid false on idle ones). sp / sm: 32-word scratch. Returns the number of
// pairs kept by stage 1 (warp-uniform).
template <class K, class F>
__device__ __forceinline__ int for_marked_pairs(uint32_t mask, int lane, int* sp, uint32_t* sm, uint16_t* q2,
                                                K&& keep, F&& eval) {
    const int cnt = __popc(mask);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) return 0;
    const unsigned lt = (1u << lane) - 1u;
    int kept_total = 0;
    sp[lane] = incl - cnt;
    sm[lane] = mask;
    __syncwarp();
    int n2 = 0;
    for (int base = 0; base < total; base += 32) {
        const int g = base + lane;
        bool kept = false;
        int pl = 0, t = 0;
        if (g < total) {
            // owner lane: the last lane whose exclusive prefix is <= g
            int src = 0;
#pragma unroll
            for (int step = 16; step; step >>= 1)
                if (sp[src + step] <= g) src += step;
            pl = src;
            t = nth_set_bit(sm[src], g - sp[src]);
            kept = keep(pl, t);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, kept);
        if (kept) q2[n2 + __popc(bal & lt)] = (uint16_t)((pl << 5) | t);
        n2 += __popc(bal);
        kept_total += __popc(bal);
        if (n2 >= 32) {
            __syncwarp();
            n2 -= 32;
            const uint16_t e = q2[n2 + lane];
            eval(true, e >> 5, e & 31);
            __syncwarp();
        }
    }
    if (n2) {
        __syncwarp();
        const bool v = lane < n2;
        const uint16_t e = v ? q2[lane] : (uint16_t)0;
        eval(v, e >> 5, e & 31);
    }
    __syncwarp();
    return kept_total;
}

// Warp-private staging of one tile of targets: position with the target's
// reach term folded into .w, axis + radius, length.
struct WarpTile {
    float4 p[kWT];
    float4 c[kWT];
    float l[kWT];
};

// One work item: probes [pfirst, pfirst + np) of one cell (cell-sorted probe
// order) against targets [tfirst, tfirst + nt) of one neighbour cell seen
// through periodic image img. pack = np | nt << 6 | image code << 15.
struct Item {
    uint32_t pfirst, tfirst, real, pack;
};

__device__ __forceinline__ void item_unpack(const Item& I, uint32_t* np, uint32_t* nt, int img[3]) {
    *np = I.pack & 63u;
    *nt = (I.pack >> 6) & 511u;
    const uint32_t im = I.pack >> 15;
    img[0] = (int)(im & 3u) - 1;
    img[1] = (int)((im >> 2) & 3u) - 1;
    img[2] = (int)((im >> 4) & 3u) - 1;
}

// Stage selector of the periodic flags: 0 = generation, 1 = contacts.
__device__ __forceinline__ int stage_per(const Real& Re, int stage) { return stage ? Re.per_con : Re.per_gen; }

constexpr int kStencilMax = 2;                                  // largest stencil radius
constexpr int kRows = (2 * kStencilMax + 1) * (2 * kStencilMax + 1);  // rows per cell

__device__ __forceinline__ void cell_xyz(const Real& Re, uint32_t c, int cc[3]) {
    const uint32_t loc = c - Re.cell_off;
    cc[0] = (int)(loc % (uint32_t)Re.n[0]);
    cc[1] = (int)((loc / (uint32_t)Re.n[0]) % (uint32_t)Re.n[1]);
    cc[2] = (int)(loc / ((uint32_t)Re.n[0] * (uint32_t)Re.n[1]));
}

// Row r = (dy, dz) of a radius-S stencil: ring 0 selects every row, ring 1
// the inner rows (|dy|, |dz| <= 1), ring 2 the others, ring 3 the centre row
// (dy = dz = 0), ring 4 the inner rows but the centre one, ring 5 the four
// inner rows next to the centre (|dy| + |dz| = 1), ring 6 the four inner
// corner rows (|dy| = |dz| = 1).
__device__ __forceinline__ bool row_in_ring(const Real& Re, int r, int ring) {
    if (ring == 0) return true;
    const int w = 2 * Re.S + 1;
    const int dy = r % w - Re.S, dz = r / w - Re.S;
    const bool inner = dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1;
    const bool centre = dy == 0 && dz == 0;
    const int ady = dy < 0 ? -dy : dy, adz = dz < 0 ? -dz : dz;
    switch (ring) {
        case 1: return inner;
        case 3: return centre;
        case 4: return inner && !centre;
        case 5: return ady + adz == 1;
        case 6: return ady == 1 && adz == 1;
        default: return !inner;
    }
}

// Items of (cell c, stencil row r) for t = c * kRows + r: probe chunks of the
// cell times target segments of every run of the row; t == ncell * kRows writes 0.
static __global__ void k_item_count(uint32_t ncell, int R, const uint32_t* __restrict__ celloff,
                                    const Real* __restrict__ reals, int stage, int ring,
                                    const uint32_t* __restrict__ pstart, const uint32_t* __restrict__ tstart,
                                    uint32_t* __restrict__ icnt) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nt27 = ncell * (uint32_t)kRows;
    if (t > nt27) return;
    if (t == nt27) { icnt[t] = 0; return; }
    const uint32_t c = t / kRows;
    const int r = (int)(t % kRows);
    const uint32_t np = pstart[c + 1] - pstart[c];
    uint32_t n = 0;
    if (np) {
        const Real& Re = reals[find_real(celloff, R, c)];
        int cc[3];
        cell_xyz(Re, c, cc);
        Run run[3];
        const int k = row_in_ring(Re, r, ring) ? stencil_row(Re, cc, r, stage_per(Re, stage), run) : 0;
        uint32_t segs = 0;
        for (int q = 0; q < k; ++q) segs += (tstart[run[q].hi + 1] - tstart[run[q].lo] + kSeg - 1) / kSeg;
        n = ((np + kWC - 1) / kWC) * segs;
    }
    icnt[t] = n;
}

// One warp per `per` consecutive (cell, row) pairs (per = 1, 2, ..., 32): the
// warp takes the pairs that have items one after the other, and lane i writes
// items i, i + 32, ... of each (item index = probe chunk * segments of the row
// + segment). With many small realisations in one launch most pairs are empty
// and per = 32 lets them cost one load and a ballot; with few, busy pairs
// per = 1 keeps one warp per pair.
static __global__ void k_item_fill(uint32_t ncell, int R, const uint32_t* __restrict__ celloff,
                                   const Real* __restrict__ reals, int stage, int ring, const uint32_t* __restrict__ pstart,
                                   const uint32_t* __restrict__ tstart, const uint32_t* __restrict__ ioff,
                                   Item* __restrict__ items, uint32_t cap, unsigned long long* __restrict__ imax,
                                   uint32_t per) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    if (gt == 0) atomicMax(imax, (unsigned long long)ioff[ncell * (uint32_t)kRows]);
    const uint32_t npair = ncell * (uint32_t)kRows;
    const uint32_t lane = gt & 31u, first = (gt >> 5) * per, t_own = first + lane;
    uint32_t k0_own = 0, kend_own = 0;
    if (lane < per && t_own < npair) { k0_own = ioff[t_own]; kend_own = ioff[t_own + 1]; }
    unsigned todo = __ballot_sync(0xffffffffu, kend_own > k0_own);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1u;
        const uint32_t t = first + (uint32_t)src;
        const uint32_t k0 = __shfl_sync(0xffffffffu, k0_own, src), kend = __shfl_sync(0xffffffffu, kend_own, src);
        const uint32_t c = t / kRows;
        const int r = (int)(t % kRows);
        const int ri = find_real(celloff, R, c);
        const Real& Re = reals[ri];
        int cc[3];
        cell_xyz(Re, c, cc);
        Run run[3];
        const int nr = row_in_ring(Re, r, ring) ? stencil_row(Re, cc, r, stage_per(Re, stage), run) : 0;
        uint32_t t0[3], nt[3], sg[3], segs = 0, im[3];
        for (int q = 0; q < nr; ++q) {
            t0[q] = tstart[run[q].lo];
            nt[q] = tstart[run[q].hi + 1] - t0[q];
            sg[q] = (nt[q] + kSeg - 1) / kSeg;
            segs += sg[q];
            im[q] = (uint32_t)(run[q].img[0] + 1) | ((uint32_t)(run[q].img[1] + 1) << 2) |
                    ((uint32_t)(run[q].img[2] + 1) << 4);
        }
        const uint32_t p0 = pstart[c], np = pstart[c + 1] - p0;
        for (uint32_t k = k0 + lane; k < kend && k < cap; k += 32) {
            const uint32_t idx = k - k0;
            const uint32_t a = (idx / segs) * kWC;
            uint32_t s = idx % segs, q = 0;
            while (s >= sg[q]) s -= sg[q++];
            const uint32_t b = s * kSeg;
            const uint32_t pa = min((uint32_t)kWC, np - a), tb = min((uint32_t)kSeg, nt[q] - b);
            items[k] = Item{p0 + a, t0[q] + b, (uint32_t)ri, pa | (tb << 6) | (im[q] << 15)};
        }
    }
}

// ---------------------------------------------------------------------------
// Exact queue: pairs the FP32 filter could not decide are appended here and
// evaluated afterwards in FP64 by full warps (on GB300 an FP64 warp
// instruction costs the same with 1 or 32 active lanes). Entry layout:
// probe (32 bits) | target (26 bits) | image of the target (3 x 2 bits).
// ---------------------------------------------------------------------------
constexpr uint32_t kXqTargetBits = 26;

__device__ __forceinline__ unsigned long long xq_pack(uint32_t probe, uint32_t target, const int img[3]) {
    uint32_t im = (uint32_t)(img[0] + 1) | ((uint32_t)(img[1] + 1) << 2) | ((uint32_t)(img[2] + 1) << 4);
    return ((unsigned long long)probe << 32) | ((unsigned long long)target << 6) | im;
}

__device__ __forceinline__ void xq_unpack(unsigned long long e, uint32_t* probe, uint32_t* target, int img[3]) {
    *probe = (uint32_t)(e >> 32);
    *target = (uint32_t)((e >> 6) & ((1u << kXqTargetBits) - 1u));
    img[0] = (int)(e & 3u) - 1;
    img[1] = (int)((e >> 2) & 3u) - 1;
    img[2] = (int)((e >> 4) & 3u) - 1;
}

// Append from divergent code: one atomic per coalesced group of lanes.
__device__ __forceinline__ void xq_push(unsigned long long* q, unsigned long long cap, unsigned long long* count,
                                        unsigned long long e) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, (unsigned long long)g.size());
    base = g.shfl(base, 0);
    unsigned long long slot = base + g.thread_rank();
    if (slot < cap) q[slot] = e;
}

// Gather rows of (pos, dir, payload) into cell-sorted order.
template <class P>
static __global__ void k_gather(uint32_t n, const uint32_t* __restrict__ ntot, const uint32_t* __restrict__ perm,
                         const float4* __restrict__ pos, const float4* __restrict__ dir, const P* __restrict__ pay,
                         float4* __restrict__ opos, float4* __restrict__ odir, P* __restrict__ opay) {
    uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t m = ntot ? *ntot : n;
    if (q >= m) return;
    uint32_t i = perm[q];
    opos[q] = pos[i];
    odir[q] = dir[i];
    opay[q] = pay[i];
}

}  // namespace nf
