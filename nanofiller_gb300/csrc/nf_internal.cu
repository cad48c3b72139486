// nf_internal.cu -- intra-rod resistor network (the `stat_conduct ... internal`
// mode of the reference): every contact end is a node on its rod; nodes of a
// rod closer than one radius merge; consecutive nodes of a rod are joined by a
// rod segment. Reference steps, restated:
//   get_node_relations            src/conductivity.cu:639-754
//   get_internal_conduct          src/conductivity.cu:756-836 (L = dt / a)
//   remove_redundant_nodes        src/adjacency_graph.cu:57-86 (merge if L <= 1)
//   reduce_node_tbl               src/adjacency_graph.cu:115-168 (mean t)
//   recalculate_segments          src/adjacency_graph.cu:170-219
//   segment admittance s0 pi a/L  tools/kirchhoff/kirchhoff.py:90-95
// Node positions are the FP64 contact parameters; the order is (rod, float(t))
// with ties in contact order, so the node table is the same on every run.
#include <cub/device/device_radix_sort.cuh>

#include "nf_engine.cuh"

namespace nf {

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

__device__ __forceinline__ uint32_t ordered_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Slot 2e: rod I at tI; slot 2e + 1: rod J at tJ (rod-rod contacts only; the
// electrode end has no node and sorts last).
__global__ void k_int_keys(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                           const double* __restrict__ t0, const double* __restrict__ t1,
                           unsigned long long* __restrict__ key, uint32_t* __restrict__ val) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    key[2 * e] = ((unsigned long long)I[e] << 32) | ordered_bits((float)t0[e]);
    val[2 * e] = 2 * e;
    key[2 * e + 1] = J[e] < NF_SNK_ELEC ? (((unsigned long long)J[e] << 32) | ordered_bits((float)t1[e]))
                                        : ~0ull;
    val[2 * e + 1] = 2 * e + 1;
}

__device__ __forceinline__ double slot_t(uint32_t slot, const double* t0, const double* t1) {
    return (slot & 1u) ? t1[slot >> 1] : t0[slot >> 1];
}

// newg[k] = 1 where sorted node k starts a node of its own (first on its rod,
// or more than one radius past its predecessor).
__global__ void k_int_flags(uint32_t nfull, const unsigned long long* __restrict__ key,
                            const uint32_t* __restrict__ val, const double* __restrict__ t0,
                            const double* __restrict__ t1, const float4* __restrict__ dir, uint32_t* __restrict__ newg) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nfull) return;
    if (k == nfull) { newg[k] = 0; return; }
    const uint32_t rod = (uint32_t)(key[k] >> 32);
    bool merged = false;
    if (k > 0 && (uint32_t)(key[k - 1] >> 32) == rod) {
        const double dt = dsub(slot_t(val[k], t0, t1), slot_t(val[k - 1], t0, t1));
        merged = ddiv(dt, (double)dir[rod].w) <= 1.0;
    }
    newg[k] = merged ? 0u : 1u;
}

// Node g = members [k, ...) of one merge group: rod and mean position (summed
// in sorted order), and the node of every contact end.
__global__ void k_int_groups(uint32_t nfull, const uint32_t* __restrict__ newg, const uint32_t* __restrict__ gid,
                             const unsigned long long* __restrict__ key, const uint32_t* __restrict__ val,
                             const double* __restrict__ t0, const double* __restrict__ t1,
                             uint32_t* __restrict__ nrod, double* __restrict__ nt, uint32_t* __restrict__ node_of_slot) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nfull) return;
    const uint32_t g = gid[k] + newg[k] - 1u;
    node_of_slot[val[k]] = g;
    if (!newg[k]) return;
    double sum = slot_t(val[k], t0, t1);
    uint32_t cnt = 1;
    for (uint32_t j = k + 1; j < nfull && !newg[j]; ++j) {
        sum = dadd(sum, slot_t(val[j], t0, t1));
        ++cnt;
    }
    nrod[g] = (uint32_t)(key[k] >> 32);
    nt[g] = ddiv(sum, (double)cnt);
}

// Contact edges between nodes (the electrode id stays as J).
__global__ void k_int_edges(uint32_t m, const uint32_t* __restrict__ J, const double* __restrict__ G,
                            const uint32_t* __restrict__ node_of_slot, uint32_t* __restrict__ eI,
                            uint32_t* __restrict__ eJ, double* __restrict__ eG) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    eI[e] = node_of_slot[2 * e];
    eJ[e] = J[e] < NF_SNK_ELEC ? node_of_slot[2 * e + 1] : J[e];
    eG[e] = G[e];
}

__global__ void k_int_segflag(uint32_t ng, const uint32_t* __restrict__ nrod, uint32_t* __restrict__ flag) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ng) return;
    flag[g] = (g + 1 < ng && nrod[g] == nrod[g + 1]) ? 1u : 0u;
}

// Rod segment between nodes g and g + 1 of one rod: L = dt / a, conductance
// sigma pi a / L.
__global__ void k_int_segs(uint32_t ng, const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                           const uint32_t* __restrict__ nrod, const double* __restrict__ nt,
                           const float4* __restrict__ dir, double sigma, uint32_t* __restrict__ eI,
                           uint32_t* __restrict__ eJ, double* __restrict__ eG, double* __restrict__ segL) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng || !flag[g]) return;
    const double a = (double)dir[nrod[g]].w;
    const double L = ddiv(dsub(nt[g + 1], nt[g]), a);
    const uint32_t s = pos[g];
    eI[s] = g;
    eJ[s] = g + 1;
    eG[s] = ddiv(dmul(dmul(sigma, 3.14159265358979323846), a), L);
    segL[s] = L;
}

// First node of every realisation (nodes are ordered by rod, rods by realisation).
__global__ void k_int_offs(uint32_t ng, const uint32_t* __restrict__ nrod, int R, const uint32_t* __restrict__ rodoff,
                           uint32_t* __restrict__ noff) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int r = find_real(rodoff, R, nrod[g]);
    if (g == 0 || find_real(rodoff, R, nrod[g - 1]) != r) noff[r] = g;
}

nf_status Engine::internal_network() {
    if (!contacts_valid) { err = "no contacts: run nf_contacts first"; return NF_ERR_STATE; }
    int_valid = false;
    const uint32_t m = (uint32_t)ct_off[R];
    const size_t n2 = 2 * (size_t)m;
    NF_CK(ikeys.ensure(n2 + 1));
    NF_CK(ikeys2.ensure(n2 + 1));
    NF_CK(ivals.ensure(n2 + 1));
    NF_CK(ivals2.ensure(n2 + 1));
    uint64_t nint = 0;
    for (int r = 0; r < R; ++r) nint += ct_int[r];
    const uint32_t nfull = (uint32_t)(m + nint);
    int_full = nfull;
    if (m) {
        NF_LAUNCH(k_int_keys, grid_for(m, 256), 256, 0, st)(m, cI.p, cJ.p, ct0.p, ct1.p, ikeys.p, ivals.p);
        NF_CK(cudaGetLastError());
        g_launches += 1;
        size_t bytes = 0;
        NF_CK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, ikeys.p, ikeys2.p, ivals.p, ivals2.p, (int)n2, 0, 64, st));
        NF_CK(cubtmp.ensure(bytes));
        NF_CK(cub::DeviceRadixSort::SortPairs(cubtmp.p, bytes, ikeys.p, ikeys2.p, ivals.p, ivals2.p, (int)n2, 0, 64,
                                              st));
    }
    NF_CK(inew.ensure(nfull + 1));
    NF_CK(igid.ensure(nfull + 1));
    NF_CK(islot.ensure(n2 + 1));
    NF_LAUNCH(k_int_flags, grid_for(nfull + 1, 256), 256, 0, st)(nfull, ikeys2.p, ivals2.p, ct0.p, ct1.p, dir.p,
                                                                 inew.p);
    NF_CK(cudaGetLastError());
    nf_status s = scan_u32(inew.p, igid.p, nfull + 1);
    if (s != NF_OK) return s;
    uint32_t ng = 0;
    NF_CK(cudaMemcpyAsync(&ng, igid.p + nfull, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    NF_CK(inrod.ensure(ng + 1));
    NF_CK(int_t.ensure(ng + 1));
    // edges: m contacts, then at most ng - 1 segments
    NF_CK(ieI.ensure((size_t)m + ng + 1));
    NF_CK(ieJ.ensure((size_t)m + ng + 1));
    NF_CK(ieG.ensure((size_t)m + ng + 1));
    NF_CK(iseg_l.ensure((size_t)ng + 1));
    if (nfull) {
        NF_LAUNCH(k_int_groups, grid_for(nfull, 256), 256, 0, st)(nfull, inew.p, igid.p, ikeys2.p, ivals2.p, ct0.p,
                                                                  ct1.p, inrod.p, int_t.p, islot.p);
        NF_CK(cudaGetLastError());
    }
    if (m) {
        NF_LAUNCH(k_int_edges, grid_for(m, 256), 256, 0, st)(m, cJ.p, cG.p, islot.p, ieI.p, ieJ.p, ieG.p);
        NF_CK(cudaGetLastError());
    }
    // segments, compacted after the contact edges
    uint32_t* sflag = inew.p;  // reuse: ng + 1 <= nfull + 1
    uint32_t* spos = igid.p;
    NF_LAUNCH(k_int_segflag, grid_for(ng + 1, 256), 256, 0, st)(ng, inrod.p, sflag);
    NF_CK(cudaGetLastError());
    s = scan_u32(sflag, spos, ng + 1);
    if (s != NF_OK) return s;
    uint32_t ns = 0;
    NF_CK(cudaMemcpyAsync(&ns, spos + ng, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (ng) {
        NF_LAUNCH(k_int_segs, grid_for(ng, 256), 256, 0, st)(ng, sflag, spos, inrod.p, int_t.p, dir.p,
                                                             prm[0].rod_sigma, ieI.p + m, ieJ.p + m, ieG.p + m,
                                                             iseg_l.p);
        NF_CK(cudaGetLastError());
    }
    // node range of every realisation
    DBuf<uint32_t>& noff = rcur;
    NF_CK(noff.ensure(R + 1));
    NF_CK(cudaMemsetAsync(noff.p, 0xff, sizeof(uint32_t) * (R + 1), st));
    if (ng) {
        NF_LAUNCH(k_int_offs, grid_for(ng, 256), 256, 0, st)(ng, inrod.p, R, rodoff.p, noff.p);
        NF_CK(cudaGetLastError());
    }
    int_off.assign(R + 1, 0);
    NF_CK(cudaMemcpyAsync(int_off.data(), noff.p, sizeof(uint32_t) * R, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    int_off[R] = ng;
    for (int r = R - 1; r >= 0; --r)
        if (int_off[r] == 0xffffffffu) int_off[r] = int_off[r + 1];
    int_count.assign(R, 0);
    for (int r = 0; r < R; ++r) int_count[r] = int_off[r + 1] - int_off[r];
    int_nodes = ng;
    int_segs = ns;
    int_edges = (uint64_t)m + ns;
    int_valid = true;
    solve_valid = false;
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
