// nf_graph.cuh -- helpers shared by the network solvers: union-find with a
// bounded walk, and deterministic block reductions (fixed thread->row mapping
// and a fixed tree).
#pragma once

namespace nf {

constexpr uint32_t kFindCap = 1u << 22;  // bound on union-find walks / CAS retries

__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x, uint32_t* err) {
    uint32_t steps = 0;
    while (true) {
        uint32_t p = parent[x];
        if (p == x) return x;
        uint32_t g = parent[p];
        if (g != p) atomicCAS(&parent[x], p, g);  // path halving
        x = p;
        if (++steps > kFindCap) { atomicExch(err, 1u); return x; }
    }
}


template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        double x = (l < NT / 32) ? sh[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (l == 0) sh[32] = x;
    }
    __syncthreads();
    return sh[32];
}

template <int NT>
__device__ __forceinline__ void block_sum2(float a, float b, double* sh, double* oa, double* ob) {
    double x = a, y = b;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_down_sync(0xffffffffu, x, o);
        y += __shfl_down_sync(0xffffffffu, y, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { sh[w] = x; sh[40 + w] = y; }
    __syncthreads();
    if (w == 0) {
        double u = (l < NT / 32) ? sh[l] : 0.0, v = (l < NT / 32) ? sh[40 + l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            u += __shfl_down_sync(0xffffffffu, u, o);
            v += __shfl_down_sync(0xffffffffu, v, o);
        }
        if (l == 0) { sh[32] = u; sh[33] = v; }
    }
    __syncthreads();
    *oa = sh[32];
    *ob = sh[33];
}

// K sums at once (K <= 4); sh holds at least 40 * K + 8 doubles.
template <int NT, int K>
__device__ __forceinline__ void block_sum_k(double* v, double* sh) {
#pragma unroll
    for (int j = 0; j < K; ++j)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0)
#pragma unroll
        for (int j = 0; j < K; ++j) sh[40 * j + w] = v[j];
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            double x = (l < NT / 32) ? sh[40 * j + l] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (l == 0) sh[40 * j + 32] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < K; ++j) v[j] = sh[40 * j + 32];
}

}  // namespace nf
