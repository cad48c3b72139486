// nf_prune.cu -- dead-end pruning: the reference's `reduce` verb
// (src/NanoFiller.cpp:71-91, reduce() src/conductivity.cu:79-138,
// contact_count_kernel_full / reductKernel inc/conductKernels.h:39-162).
//
// The reference counts, for every rod, its contacts within the tunnelling
// cutoff (electrode buffer-layer rods included, no screening), deletes every
// rod outside the electrode layers with fewer than min_cont (2) of them, and
// repeats until a pass deletes nothing. The rods left are the min_cont-core
// of the contact graph with the electrodes kept, which is unique whatever the
// order of deletion; dangling trees and isolated rods carry no current, so the
// network's G_eff is unchanged.
//
// GB300 form: one contact sweep (the contact extraction with screening off),
// then peeling rounds over the contact list on the device -- a degree count
// and a threshold pass per round, one 4-byte read-back per round -- and a
// stable compaction of the surviving rods (stream order kept) followed by a
// rebuild of the cell lists.
#include <vector>

#include "nf_engine.cuh"

namespace nf {

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

// Contacts of alive rods with alive rods or an electrode, per rod.
__global__ void k_prune_deg(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                            const uint32_t* __restrict__ alive, uint32_t* __restrict__ deg) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const uint32_t i = I[e], j = J[e];
    if (!alive[i]) return;
    if (j >= NF_SNK_ELEC) {
        atomicAdd(&deg[i], 1u);
    } else if (alive[j]) {
        atomicAdd(&deg[i], 1u);
        atomicAdd(&deg[j], 1u);
    }
}

// Alive rods below the threshold go, all in the same pass.
__global__ void k_prune_mark(uint32_t n, uint32_t k, const uint32_t* __restrict__ deg, uint32_t* __restrict__ alive,
                             uint32_t* __restrict__ removed) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !alive[i] || deg[i] >= k) return;
    alive[i] = 0;
    atomicAdd(removed, 1u);
}

__global__ void k_prune_gather(uint32_t n, const uint32_t* __restrict__ alive, const uint32_t* __restrict__ pos_of,
                               const float4* __restrict__ p, const float4* __restrict__ d,
                               const uint64_t* __restrict__ s, float4* __restrict__ p2, float4* __restrict__ d2,
                               uint64_t* __restrict__ s2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !alive[i]) return;
    const uint32_t q = pos_of[i];
    p2[q] = p[i];
    d2[q] = d[i];
    s2[q] = s[i];
}

nf_status Engine::compact_rods(const uint32_t* keepf, uint32_t n, uint32_t left) {
    if (R != 1) { err = "rod compaction runs on a single-realisation handle"; return NF_ERR_STATE; }
    DBuf<uint32_t> posn;
    NF_CK(posn.ensure(n + 1));
    nf_status s = scan_u32(keepf, posn.p, n + 1);
    if (s != NF_OK) return s;
    DBuf<float4> p2, d2;
    DBuf<uint64_t> s2;
    NF_CK(p2.ensure(left + 1));
    NF_CK(d2.ensure(left + 1));
    NF_CK(s2.ensure(left + 1));
    if (n)
        NF_LAUNCH(k_prune_gather, grid_for(n, 256), 256, 0, st)(n, keepf, posn.p, pos.p, dir.p, sidx.p, p2.p, d2.p,
                                                               s2.p);
    NF_CK(cudaGetLastError());
    if (left) {
        NF_CK(cudaMemcpyAsync(pos.p, p2.p, sizeof(float4) * left, cudaMemcpyDeviceToDevice, st));
        NF_CK(cudaMemcpyAsync(dir.p, d2.p, sizeof(float4) * left, cudaMemcpyDeviceToDevice, st));
        NF_CK(cudaMemcpyAsync(sidx.p, s2.p, sizeof(uint64_t) * left, cudaMemcpyDeviceToDevice, st));
    }
    count[0] = left;
    NF_CK(cudaMemcpyAsync(dcount.p, count.data(), sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    // the temporaries are freed on return: finish their use first
    NF_CK(cudaStreamSynchronize(st));
    return rebuild_cells();
}

nf_status Engine::prune(int min_cont, nf_reduce_stats* out) {
    if (R != 1) { err = "pruning runs on a single-realisation handle"; return NF_ERR_STATE; }
    if (min_cont < 0) return NF_ERR_PARAM;
    EventPair ev;
    NF_CK(ev.create());
    NF_CK(cudaEventRecord(ev.a, st));
    // contacts within the cutoff, unscreened (the reference counts them all)
    const int32_t screening = prm[0].screening;
    prm[0].screening = 0;
    nf_status s = contacts();
    prm[0].screening = screening;
    if (s != NF_OK) return s;
    const uint32_t n = count[0];
    const uint32_t m = (uint32_t)ct_off[1];
    DBuf<uint32_t> alive, deg, ctr1;
    NF_CK(alive.ensure(n + 1));
    NF_CK(deg.ensure(n + 1));
    NF_CK(ctr1.ensure(1));
    // every rod starts alive
    std::vector<uint32_t> ones(n + 1, 1u);
    ones[n] = 0;
    NF_CK(cudaMemcpyAsync(alive.p, ones.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, st));
    int rounds = 0;
    uint32_t left = n;
    while (n) {
        NF_CK(cudaMemsetAsync(deg.p, 0, sizeof(uint32_t) * (n + 1), st));
        NF_CK(cudaMemsetAsync(ctr1.p, 0, sizeof(uint32_t), st));
        if (m) NF_LAUNCH(k_prune_deg, grid_for(m, 256), 256, 0, st)(m, cI.p, cJ.p, alive.p, deg.p);
        NF_LAUNCH(k_prune_mark, grid_for(n, 256), 256, 0, st)(n, (uint32_t)min_cont, deg.p, alive.p, ctr1.p);
        NF_CK(cudaGetLastError());
        uint32_t removed = 0;
        NF_CK(cudaMemcpyAsync(&removed, ctr1.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        NF_CK(cudaStreamSynchronize(st));
        if (removed == 0) break;
        left -= removed;
        ++rounds;
    }
    // stable compaction of the survivors
    if (left < n) {
        s = compact_rods(alive.p, n, left);
        if (s != NF_OK) return s;
    }
    contacts_valid = false;
    solve_valid = false;
    int_valid = false;
    NF_CK(cudaEventRecord(ev.b, st));
    NF_CK(cudaEventSynchronize(ev.b));
    float ms = 0;
    NF_CK(cudaEventElapsedTime(&ms, ev.a, ev.b));
    if (out) {
        out->rods_before = n;
        out->rods_after = left;
        out->contacts = m;
        out->rounds = rounds;
        out->min_contacts = min_cont;
        out->ms = ms;
    }
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
