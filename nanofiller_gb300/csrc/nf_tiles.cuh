// nf_tiles.cuh -- work decomposition of the cell-pair kernels.
//
// Probes (candidates, rods or virtual rods) are binned by cell (CSR pstart).
// A chunk is up to kWC = 32 probes of one cell, one per lane of a warp; a warp
// of the pair kernels takes one (chunk, stencil offset) pair: it owns one
// neighbour cell of one probe chunk, stages that cell's targets 32 at a time
// in a warp-private shared-memory tile (one coalesced load per lane), and
// every lane tests its probe against each staged target (all lanes read the
// same shared-memory word: broadcast, no bank conflict). Warps only meet at
// __syncwarp, so a warp whose cell is sparse or whose probes are all decided
// retires without waiting for the other warps of its block. The 27 offsets of
// a chunk run as 27 independent warps, so a dense cell fills many SMs.
#pragma once
#include <cstdint>

#include <cooperative_groups.h>

#include "nf_common.cuh"

namespace nf {

constexpr int kTPB = 128;   // threads per block of the pair kernels (4 independent warps)
constexpr int kWC = 32;     // probes per chunk: one warp per (chunk, neighbour cell)
constexpr int kWT = 32;     // targets per warp-private shared-memory tile

// Warp-private staging of one tile of targets: position with the target's
// sphere term folded into .w (l/2 + a + eps + a*scf), axis + radius, length.
struct WarpTile {
    float4 p[kWT];
    float4 c[kWT];
    float l[kWT];
};

struct Chunk {
    uint32_t cell;   // global cell id of the probes
    uint32_t first;  // first probe (index into the cell-sorted probe order)
    uint32_t n;      // probes in the chunk (<= kWC)
    uint32_t real;   // realisation of the cell
};

// Number of chunks per cell.
static __global__ void k_chunk_count(uint32_t ncell, const uint32_t* __restrict__ pstart, uint32_t* __restrict__ nch) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > ncell) return;
    if (c == ncell) { nch[c] = 0; return; }
    uint32_t n = pstart[c + 1] - pstart[c];
    nch[c] = (n + kWC - 1) / kWC;
}

static __global__ void k_chunk_fill(uint32_t ncell, int R, const uint32_t* __restrict__ celloff,
                             const uint32_t* __restrict__ pstart, const uint32_t* __restrict__ choff,
                             Chunk* __restrict__ chunks) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    uint32_t b = pstart[c], n = pstart[c + 1] - b, k0 = choff[c];
    uint32_t r = (uint32_t)find_real(celloff, R, c);
    for (uint32_t k = 0; k * kWC < n; ++k) {
        Chunk ch;
        ch.cell = c;
        ch.first = b + k * kWC;
        ch.n = min((uint32_t)kWC, n - k * kWC);
        ch.real = r;
        chunks[k0 + k] = ch;
    }
}

// Decode the stencil neighbour of chunk cell `cell` (global id) for offset o.
__device__ __forceinline__ bool chunk_neighbour(const Real& Re, uint32_t cell, int o, int per, uint32_t* nc,
                                                int img[3]) {
    uint32_t loc = cell - Re.cell_off;
    int c[3];
    c[0] = (int)(loc % (uint32_t)Re.n[0]);
    c[1] = (int)((loc / (uint32_t)Re.n[0]) % (uint32_t)Re.n[1]);
    c[2] = (int)(loc / ((uint32_t)Re.n[0] * (uint32_t)Re.n[1]));
    return stencil(Re, c, o, per, nc, img);
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
