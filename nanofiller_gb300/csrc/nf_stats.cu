// nf_stats.cu -- statistics of the rod set and its contacts: the reference's
// stat_nematic, stat_phitheta, stat_mutangle and stat_contacts verbs
// (src/NanoFiller.cpp:92-121, src/statistics_collection.cu:463-864) and its
// write_ort / write_lmp writers (src/IO.cpp:77-146).
//
// The reference gathers these with its own cell-stride sweeps; here they are
// reductions over the rod arrays and over the (unscreened) contact list that
// the contact extraction already produces:
//   nematic order   S = sum_i P2(c_i . n) / N, rods with a direction component
//                   <= -1 + 1e-6 left out of the sum but not of N
//                   (nematic_func, statistics_collection.cu:589-614)
//   phi-theta       theta = acos(cz), phi = acos(cx / sqrt(1 - cz^2)) for
//                   theta in (1e-3, pi - 1e-3) else 0, bins of pi / nbins
//                   (statKernel_ANGL, inc/statKernel_ANGL.h:57-63)
//   mutual angle    pairs whose closest points are interior to both rods and
//                   whose axis gap D - a_i - a_j is below STAT_DIST_LIM, binned
//                   by acos|c_i . c_j| in steps of (pi + TOL) / 2 / nbins
//                   (statKernel_MUT_ANGLE_weightedFloat, inc/statKernel_MUT.h:26-131)
//   contacts per rod  rod-rod contacts within STAT_DIST_LIM counted at both
//                   ends (statKernel_CntctPerInc, inc/statKernel_MUT.h:452-512)
// Histograms use integer atomics (exact, order-free); the nematic sum is FP64
// per block, added in block order on the host.
#include <cmath>
#include <vector>

#include "nf_engine.cuh"

namespace nf {

#define NF_CK(x)                                            \
    do {                                                    \
        cudaError_t e_ = (x);                               \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);    \
    } while (0)

static inline unsigned grid_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

constexpr int kStatTPB = 256;

__global__ void k_nematic(uint32_t n, const float4* __restrict__ dir, double ax, double ay, double az,
                          double* __restrict__ part) {
    __shared__ double sh[kStatTPB];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (i < n) {
        const float4 c = dir[i];
        const float lim = -1.0f + 1.0e-6f;
        if (c.x > lim && c.y > lim && c.z > lim) {
            const double ct = dadd(dadd(dmul(ax, (double)c.x), dmul(ay, (double)c.y)), dmul(az, (double)c.z));
            v = ddiv(dsub(dmul(3.0, dmul(ct, ct)), 1.0), 2.0);
        }
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = kStatTPB / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = dadd(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_phitheta(uint32_t n, const float4* __restrict__ dir, int bx, int by,
                           unsigned long long* __restrict__ hist) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 c = dir[i];
    const double pi = 3.14159265358979323846;
    const double cz = fmin(fmax((double)c.z, -1.0), 1.0);
    const double theta = acos(cz);
    double phi = 0.0;
    if (theta > 1e-3 && theta < pi - 1e-3) {
        const double q = ddiv((double)c.x, sqrt(dsub(1.0, dmul(cz, cz))));
        phi = acos(fmin(fmax(q, -1.0), 1.0));
    }
    int ip = (int)floor(ddiv(phi, ddiv(pi, (double)bx)));
    int it = (int)floor(ddiv(theta, ddiv(pi, (double)by)));
    ip = ip < 0 ? 0 : (ip >= bx ? bx - 1 : ip);  // phi = pi or theta = pi fall in the last bin
    it = it < 0 ? 0 : (it >= by ? by - 1 : it);
    atomicAdd(&hist[ip + it * bx], 1ull);
}

// Rod-rod contacts: per-rod counts, and the mutual-angle histogram of pairs
// with interior closest points and axis gap below the limit.
__global__ void k_pair_stats(uint32_t m, const uint32_t* __restrict__ I, const uint32_t* __restrict__ J,
                             const double* __restrict__ t0, const double* __restrict__ t1,
                             const double* __restrict__ D, const float4* __restrict__ pos,
                             const float4* __restrict__ dir, double lim, double step, int bins,
                             uint32_t* __restrict__ per_rod, unsigned long long* __restrict__ hist) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= m) return;
    const uint32_t i = I[e], j = J[e];
    if (j >= NF_SNK_ELEC) return;
    atomicAdd(&per_rod[i], 1u);
    atomicAdd(&per_rod[j], 1u);
    const float4 ci = dir[i], cj = dir[j];
    const double hi = ddiv((double)pos[i].w, 2.0), hj = ddiv((double)pos[j].w, 2.0);
    const bool interior = fabs(t0[e]) < hi && fabs(t1[e]) < hj;
    if (!interior || !(dsub(dsub(D[e], (double)ci.w), (double)cj.w) < lim)) return;
    const double dot = dadd(dadd(dmul((double)ci.x, (double)cj.x), dmul((double)ci.y, (double)cj.y)),
                            dmul((double)ci.z, (double)cj.z));
    const double g = acos(fmin(fabs(dot), 1.0));
    const int b = ((int)floor(ddiv(g, step))) % bins;
    atomicAdd(&hist[b], 1ull);
}

nf_status Engine::unscreened_contacts(bool* recomputed) {
    *recomputed = false;
    if (contacts_valid && !contacts_screened) return NF_OK;
    const int32_t screening = prm[0].screening;
    prm[0].screening = 0;
    nf_status s = contacts();
    prm[0].screening = screening;
    *recomputed = true;
    return s;
}

nf_status Engine::stat_nematic(const double axis[3], double* S) {
    if (R != 1) { err = "statistics run on a single-realisation handle"; return NF_ERR_STATE; }
    const uint32_t n = count[0];
    const double nrm = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
    if (!(nrm > 0)) return NF_ERR_PARAM;
    if (n == 0) { *S = 0.0; return NF_OK; }
    const unsigned nb = grid_for(n, kStatTPB);
    DBuf<double> part;
    NF_CK(part.ensure(nb));
    NF_LAUNCH(k_nematic, nb, kStatTPB, 0, st)(n, dir.p, axis[0] / nrm, axis[1] / nrm, axis[2] / nrm, part.p);
    NF_CK(cudaGetLastError());
    std::vector<double> h(nb);
    NF_CK(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    double sum = 0.0;
    for (double v : h) sum += v;
    *S = sum / n;
    return NF_OK;
}

nf_status Engine::stat_phitheta(int bx, int by, uint64_t* hist) {
    if (R != 1) { err = "statistics run on a single-realisation handle"; return NF_ERR_STATE; }
    if (bx <= 0 || by <= 0 || bx > 4096 || by > 4096) return NF_ERR_PARAM;
    const uint32_t n = count[0];
    DBuf<unsigned long long> d;
    NF_CK(d.ensure((size_t)bx * by));
    NF_CK(cudaMemsetAsync(d.p, 0, sizeof(unsigned long long) * bx * by, st));
    if (n) NF_LAUNCH(k_phitheta, grid_for(n, 256), 256, 0, st)(n, dir.p, bx, by, d.p);
    NF_CK(cudaGetLastError());
    NF_CK(cudaMemcpyAsync(hist, d.p, sizeof(unsigned long long) * bx * by, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    return NF_OK;
}

nf_status Engine::stat_pairs(int bins, uint64_t* hist, uint32_t* per_rod, size_t capacity, nf_pair_stats* out) {
    if (R != 1) { err = "statistics run on a single-realisation handle"; return NF_ERR_STATE; }
    if (bins <= 0 || bins > 1 << 20) return NF_ERR_PARAM;
    const uint32_t n = count[0];
    if (per_rod && capacity < n) { err = "per-rod buffer too small"; return NF_ERR_CAPACITY; }
    bool recomputed = false;
    nf_status s = unscreened_contacts(&recomputed);
    if (s != NF_OK) return s;
    const uint32_t m = (uint32_t)ct_off[1];
    DBuf<unsigned long long> dh;
    DBuf<uint32_t> dp;
    NF_CK(dh.ensure(bins));
    NF_CK(dp.ensure(n + 1));
    NF_CK(cudaMemsetAsync(dh.p, 0, sizeof(unsigned long long) * bins, st));
    NF_CK(cudaMemsetAsync(dp.p, 0, sizeof(uint32_t) * (n + 1), st));
    const double lim = (double)prm[0].stat_dist_lim;
    const double step = ((3.14159265358979323846 + (double)prm[0].tol) / 2.0) / bins;
    if (m)
        NF_LAUNCH(k_pair_stats, grid_for(m, 256), 256, 0, st)(m, cI.p, cJ.p, ct0.p, ct1.p, cD.p, pos.p, dir.p, lim,
                                                             step, bins, dp.p, dh.p);
    NF_CK(cudaGetLastError());
    std::vector<uint32_t> hp(n);
    std::vector<unsigned long long> hh(bins);
    if (n) NF_CK(cudaMemcpyAsync(hp.data(), dp.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaMemcpyAsync(hh.data(), dh.p, sizeof(unsigned long long) * bins, cudaMemcpyDeviceToHost, st));
    NF_CK(cudaStreamSynchronize(st));
    nf_pair_stats o{};
    o.rods = n;
    uint64_t total = 0;
    uint32_t mx = 0;
    for (uint32_t i = 0; i < n; ++i) { total += hp[i]; mx = hp[i] > mx ? hp[i] : mx; }
    o.contacts_total = total;
    o.pairs = total / 2;
    o.max_per_rod = mx;
    o.mean_per_rod = n ? (double)total / n : 0.0;
    uint64_t hs = 0;
    for (int b = 0; b < bins; ++b) { if (hist) hist[b] = hh[b]; hs += hh[b]; }
    o.angle_pairs = hs;
    if (per_rod) for (uint32_t i = 0; i < n; ++i) per_rod[i] = hp[i];
    if (out) *out = o;
    if (recomputed && prm[0].screening) {  // the handle's own contacts are screened ones
        contacts_valid = false;
        solve_valid = false;
        int_valid = false;
    }
    return NF_OK;
}

#undef NF_CK
}  // namespace nf
