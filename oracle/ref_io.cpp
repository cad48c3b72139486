// ref_io.cpp -- host wrapper around the reference's own file writers and
// readers (TEST INFRASTRUCTURE). oracle/ref_build.sh compiles it with -I
// pointing at the reference's inc/ and src/ directories: src/IO.cpp and
// src/stateSR.cpp are compiled in place, nothing of them is copied. The
// outputs become fixtures (tests/golden/ref_formats.npz) that pin the
// library's writers byte for byte.
#include <cstdlib>
#include <cstring>
#include <cuda_runtime.h>

#include "IO.cpp"
#include "stateSR.cpp"

// Host stand-ins for the CUDA runtime calls the writers make: their "device"
// arrays are host arrays here. No CUDA library is linked.
extern "C" cudaError_t cudaMemcpy(void* dst, const void* src, size_t n, cudaMemcpyKind) {
    std::memcpy(dst, src, n);
    return cudaSuccess;
}
extern "C" cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::malloc(n ? n : 1);
    return cudaSuccess;
}
extern "C" cudaError_t cudaGetLastError(void) { return cudaSuccess; }
extern "C" const char* cudaGetErrorString(cudaError_t) { return "no error"; }

// The parameter object's members the writers touch are set by the wrappers
// below; its own constructor, destructor and device set-up (src/simPrms.cpp)
// are not part of the file formats.
simPrms::simPrms() {}
simPrms::~simPrms(void) {}
int simPrms::device_config(void) { return 1; }

namespace {
void to_cnt(int n, const float* rods9, CNT_t* out) {  // rods9: x y z cx cy cz l a k per rod
    for (int i = 0; i < n; ++i) {
        const float* r = rods9 + 9 * i;
        out[i].r = make_float3(r[0], r[1], r[2]);
        out[i].c = make_float3(r[3], r[4], r[5]);
        out[i].l = r[6];
        out[i].a = r[7];
        out[i].k = r[8];
    }
}
}  // namespace

extern "C" {

// write_CNTvtk / write_CNT_ORTvtk / write_CNTlmp (src/IO.cpp:38-146); the
// writers prepend "./" and append their extension to `base`.
int ref_write_vtk(const char* base, int n, const float* rods9) {
    CNT_t* a = new CNT_t[n > 0 ? n : 1];
    to_cnt(n, rods9, a);
    write_CNTvtk(base, n, a);
    delete[] a;
    return 0;
}
int ref_write_ort_vtk(const char* base, int n, const float* rods9) {
    CNT_t* a = new CNT_t[n > 0 ? n : 1];
    to_cnt(n, rods9, a);
    write_CNT_ORTvtk(base, n, a);
    delete[] a;
    return 0;
}
int ref_write_lmp(const char* base, int n, const float* rods9, const float* box, float density) {
    CNT_t* a = new CNT_t[n > 0 ? n : 1];
    to_cnt(n, rods9, a);
    float b[3] = {box[0], box[1], box[2]};
    write_CNTlmp(base, n, a, b, density);
    delete[] a;
    return 0;
}

// save_state_BIN (src/stateSR.cpp:54-89) of a state given as header fields and
// host arrays (occ, addr: ext cells; planes: 9 x ttl floats).
int ref_save_state(const char* path, const float* phys, const float* edge, const int* ext, float l, float a, int ttl,
                   int num, float tol, const short* occ, const int* addr, const float* planes) {
    simPrms S;
    for (int d = 0; d < 3; ++d) {
        S.physDim[d] = phys[d];
        S.Domains.edge[d] = edge[d];
        S.Domains.ext[d] = ext[d];
    }
    S.l = l;
    S.a = a;
    S.Domains.ttlCNT = ttl;
    S.numCNT = num;
    S.TOL = tol;
    S.Domains.d_dmnOcc = const_cast<short*>(occ);
    S.Domains.d_dmnAddr = const_cast<int*>(addr);
    S.d_result = const_cast<float*>(planes);
    save_state_BIN(path, S);
    return 0;
}

// read_state_BIN (src/stateSR.cpp:90-134): header fields and the arrays it read.
int ref_read_state(const char* path, float* phys, float* edge, int* ext, float* l, float* a, int* ttl, int* num,
                   float* tol, short* occ, int* addr, float* planes, int cells_cap, int planes_cap) {
    simPrms S;
    S.Domains.d_dmnOcc = nullptr;
    S.Domains.d_dmnAddr = nullptr;
    S.d_result = nullptr;
    read_state_BIN(path, &S);
    for (int d = 0; d < 3; ++d) {
        phys[d] = S.physDim[d];
        edge[d] = S.Domains.edge[d];
        ext[d] = S.Domains.ext[d];
    }
    *l = S.l;
    *a = S.a;
    *ttl = S.Domains.ttlCNT;
    *num = S.numCNT;
    *tol = S.TOL;
    const int cells = S.Domains.ext[0] * S.Domains.ext[1] * S.Domains.ext[2];
    if (cells > cells_cap || 9 * S.Domains.ttlCNT > planes_cap) return -1;
    std::memcpy(occ, S.Domains.d_dmnOcc, sizeof(short) * cells);
    std::memcpy(addr, S.Domains.d_dmnAddr, sizeof(int) * cells);
    std::memcpy(planes, S.d_result, sizeof(float) * 9 * S.Domains.ttlCNT);
    return 0;
}

}  // extern "C"
