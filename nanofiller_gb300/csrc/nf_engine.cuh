// nf_engine.cuh -- per-handle device state of the GB300 path and the stage
// entry points (generation, contacts, network solve, adjoint).
//
// Memory layout in HBM (all realisations of a batch side by side):
//   rods   pos[N] float4 (x,y,z,l), dir[N] float4 (cx,cy,cz,a): 32 B per rod,
//          SoA so a warp reads 512 contiguous bytes per field pair;
//          realisation r owns slots [rod_off_r, rod_off_r + target_r).
//   cells  one global cell index space; realisation r owns
//          [cell_off_r, cell_off_r + ncell_r). A CSR (rstart) over the
//          cell-sorted copy spos/sdir/sid is rebuilt by a counting sort
//          (count, exclusive scan, scatter) after every round.
//   round  candidates of one round are compacted (stream order) and binned by
//          cell the same way; per-candidate state + a fixed-capacity list of
//          earlier conflicting candidates.
#pragma once
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/nanofiller_gb300.h"
#include "nf_common.cuh"
#include "nf_tiles.cuh"
#include "nf_tube.cuh"

namespace nf {

constexpr int kConflictCap = 32;  // earlier in-round conflicts kept per candidate

enum CandState : uint8_t { ST_NONE = 0, ST_REJ_OLD = 1, ST_ALIVE = 2, ST_ACC = 3, ST_REJ_CONF = 4 };

// Device counters (unsigned long long) in Engine::ctr.
enum Ctr {
    C_PAIR_TESTS = 0, C_EXACT, C_FLIPS, C_OVERFLOW, C_UNDECIDED,
    C_CT_PAIRS, C_CT_EXACT, C_CT_FLIPS, C_CT_RECORDS, C_SCR_PAIRS, C_SCR_EXACT,
    C_CG_ITERS, C_XQ_OLD, C_XQ_CONF, C_XQ, C_CERT, C_ITEMS, C_G_ITEMS, C_G_TILES, C_G_MARKED, C_G_LINE, C_XQ_MARK,
    C_TUBE_OVF, C_TROD_OVF, C_NCTR
};

// Device memory of the library's buffers (nf_alloc.cu): blocks come from a
// process-wide cache of freed blocks (per device, sizes rounded up to four
// classes per power of two) before cudaMalloc; a freed block returns to the
// cache after the device has finished the work that may still use it.
// *bytes is rounded up to the block's size.
cudaError_t dev_alloc(void** p, size_t* bytes);
void dev_free(void* p, size_t bytes);

// Device buffer owned by its object: released by release() or the destructor.
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t cap = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    cudaError_t ensure(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        release();
        size_t bytes = (n < 1 ? 1 : n) * sizeof(T);
        cudaError_t e = dev_alloc((void**)&p, &bytes);
        if (e == cudaSuccess) cap = bytes / sizeof(T);
        else p = nullptr;
        return e;
    }
    void release() {
        if (p) dev_free(p, cap * sizeof(T));
        p = nullptr;
        cap = 0;
    }
};

// Reverse Cuthill-McKee order of a symmetric sparse graph given as CSR rows
// plus chain links i -> i + 1 where up[i]: perm[old] = new; returns the
// bandwidth of the reordered graph.
uint32_t rcm_order(uint32_t n, const std::vector<uint32_t>& rowp, const std::vector<uint32_t>& col,
                   const std::vector<char>& up, std::vector<uint32_t>* perm);

// Two CUDA events, destroyed with the object (early returns included).
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t create() {
        cudaError_t e = cudaEventCreate(&a);
        return e == cudaSuccess ? cudaEventCreate(&b) : e;
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// One contact record before sorting / screening (64 B).
struct Rec {
    uint32_t i, j;      // global rod slots, i < j
    int8_t img[4];      // image of j (x,y,z), pad
    uint32_t flags;     // bit0: screened
    double t0, t1, d, Dx, u0, u1;
};

// Per-kernel CUDA-event timing on the launching stream (diagnostic, off by default).
enum KT { KT_STREAM = 0, KT_OLD, KT_CONF, KT_RESOLVE, KT_CTPAIRS, KT_SCREEN, KT_CG, KT_N };
struct KTime {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev;
    double ms = 0, bytes = 0, flops = 0;
    uint64_t n = 0;
};

struct Engine {
    cudaStream_t st = 0;
    bool timing = false;
    KTime kt[KT_N];
    std::vector<cudaEvent_t> evpool;
    cudaEvent_t tev();
    void tstart(int k) { if (timing) kt[k].ev.push_back({tev(), nullptr}), cudaEventRecord(kt[k].ev.back().first, st); }
    void tstop(int k) { if (timing) { kt[k].ev.back().second = tev(); cudaEventRecord(kt[k].ev.back().second, st); kt[k].n++; } }
    void tbytes(int k, double b, double f) { if (timing) { kt[k].bytes += b; kt[k].flops += f; } }
    nf_status tresolve();
    int dev = 0;
    int nsm = 0;
    std::string err;

    // realisations
    int R = 0;
    std::vector<nf_params> prm;
    std::vector<Real> hreal;
    DBuf<Real> dreal;
    std::vector<std::vector<float>> hmesh;  // host copies of meshes (per realisation, may be empty)
    DBuf<float> mesh;
    bool mesh_dirty = true;  // host meshes changed since the last upload
    uint32_t ncell = 0;

    // rods
    std::vector<uint32_t> count;     // accepted per realisation (host mirror)
    std::vector<uint64_t> knext;     // next stream index per realisation
    std::vector<uint64_t> drawn;     // stream indices consumed
    std::vector<uint64_t> dens_acc;  // density-accepted up to the stop
    std::vector<int> rounds_r;
    uint64_t rod_slots = 0;
    DBuf<float4> pos, dir;
    DBuf<uint64_t> sidx;
    DBuf<uint32_t> dcount;  // device copy of count
    DBuf<uint32_t> rodoff;  // R+1 prefix of targets
    DBuf<uint32_t> rstart, rcursor;
    DBuf<float4> spos, sdir;
    DBuf<uint32_t> sid;
    bool cells_valid = false;

    // round scratch
    DBuf<uint32_t> coff, keep, kpos, ccount, cstart, ccursor, cperm, creal, ccell, ccnt, clist, accf, accpos;
    DBuf<uint64_t> kbeg, csidx;
    DBuf<float4> cpos, cdir;
    DBuf<float4> gpos, gdir;     // candidates in cell order
    DBuf<float4> apos, adir;     // survivors of the old-rod test in cell order
    DBuf<uint32_t> aperm, astart;
    DBuf<Item> items;            // work list of the pair kernels
    size_t it_cap = 1 << 20;     // its capacity (grown on overflow)
    DBuf<unsigned long long> xq, xq2;  // exact queues (pairs left to FP64)
    DBuf<uint32_t> xqc;                // tube cell of each contact-queue entry
    size_t xq_cap = 1 << 16;
    DBuf<uint32_t> icnt, ioff, celloff;
    DBuf<uint8_t> state;
    DBuf<uint32_t> meta;   // per-realisation round metadata
    DBuf<unsigned long long> ctr;
    DBuf<unsigned char> cubtmp;
    DBuf<uint32_t> u32tmp;

    // tube grid of the pair sweeps (nf_tube.cuh): registrations of the placed
    // rods (trod*), of the round's candidates or survivors (tcnd*), per-cell
    // CSR over ntcell cells, and the work list of a tube sweep
    bool tube = false;
    uint32_t ntcell = 0;
    int trod_stage = -1;                    // stage of the current rod registrations (-1: stale)
    bool trod_append = false;               // rods appended since the stage 0 registration
    bool trod_room = false;                 // that registration left room in its cells
    std::vector<uint32_t> trod_nreg;        // per realisation: rods in the registration
    DBuf<uint32_t> trod_dnreg;              // the same on the device (the append's first rod)
    DBuf<float> trod_grow;                  // per realisation: growth expected after the registration
    DBuf<uint32_t> toffs;                   // R + 1 prefix of tube cells
    DBuf<uint32_t> trod_start, trod_cur, trod_ent;
    DBuf<uint32_t> tcnd_start, tcnd_cur, tcnd_ent, tcnd_cnt;
    DBuf<float4> trod_pos, trod_dir, tcnd_pos, tcnd_dir;  // each entry's object geometry
    DBuf<TItem> titems;
    size_t tit_cap = 1 << 20;
    uint32_t tit_nseg = 0;  // cell segments of the last tube_items (its item count sits at tioff[tit_nseg])
    size_t trod_total = 0, tcnd_total = 0;  // entries of the last rod / candidate (or virtual rod) registration
    DBuf<uint32_t> tioff;

    // contacts
    DBuf<Rec> rec, rec2;
    DBuf<uint32_t> rcnt, rpos, rcur;
    DBuf<unsigned long long> recn;
    size_t n_int = 0, n_snk = 0, n_src = 0, n_scr = 0;
    DBuf<uint32_t> cI, cJ;       // final contacts (global slots; J may be an electrode id)
    DBuf<double> ct0, ct1, cD, cG, cS;
    DBuf<int8_t> cimg;
    DBuf<uint32_t> creal2;       // realisation of each final contact
    std::vector<uint64_t> ct_off;  // per realisation prefix of final contacts (host)
    std::vector<uint64_t> ct_int, ct_snk, ct_src, ct_scr;
    bool contacts_valid = false;
    bool contacts_screened = false;  // the current list had screened contacts removed
    DBuf<uint32_t> eflag;
    // virtual rods of the screening test: FP32 copies for the filter, FP64
    // record (x,y,z,cx,cy,cz,l,a, wrap shift x,y,z), cell binning
    DBuf<float4> vpf, vdf;
    DBuf<double> vdbl;
    DBuf<uint32_t> vcell, vperm, vstart, vcur;

    // solve
    DBuf<double> vsrc, vsnk, volt;
    DBuf<uint32_t> parent, cflag, aidx, rowp, col, deg;
    DBuf<float> val32, diag32, chain32;
    DBuf<double> val64, diag64, bvec, xvec, cdiag, chain64;
    DBuf<double> valC64, diagC64, cdiagC, bvecC;  // capacitive parts (admittance form)
    DBuf<double> acG, acC, acchi;                 // scaled edge admittances of an AC call, start chi
    DBuf<uint32_t> ecnt, eoff, elist;             // electrode edges per node (network assembly)
    DBuf<float> cgbuf;
    DBuf<double> cgred;
    DBuf<double> dcband, dcwork;   // banded factors and solve vectors of the direct DC form
    DBuf<uint32_t> dcperm;         // per-realisation RCM order (local indices)
    DBuf<unsigned long long> dcboff;  // band offset per realisation
    DBuf<uint32_t> dcbw;           // bandwidth per realisation
    DBuf<double> bcrbuf;           // block cyclic reduction: blocks, then solve vectors
    DBuf<uint32_t> bcroff;         // first block per realisation
    DBuf<double> cgout;            // per-realisation solve results (CgOut records)
    DBuf<uint32_t> asmoff;         // assembly read-back: node offsets, then active bases and the error word
    std::vector<nf_solve_stats> solve_st;
    bool solve_valid = false;

    // adaptive generation (single realisation): per-cell orientation laws,
    // their tensor sums, and the clusterisation neighbour lists
    std::vector<float> hlaw;        // kLawF floats per law cell (host mirror)
    std::vector<double> hlawd;      // kLawD doubles per law cell (host mirror)
    DBuf<float> law;
    DBuf<double> lawd;
    DBuf<unsigned long long> lacc;  // 7 fixed-point sums per law cell
    int32_t lawn[3] = {0, 0, 0};
    bool laws_set = false;          // hlaw holds the laws of the last generation
    DBuf<uint32_t> clu_cnt, clu_off, clu_snaps;
    DBuf<unsigned long long> clu_key, clu_key2;
    uint64_t ad_epochs = 0, ad_refits = 0, ad_thinned = 0, ad_snapped = 0;

    // stats
    nf_gen_stats gst{};
    nf_contact_stats cst{};

    // --- set-up ------------------------------------------------------------
    nf_status init(const nf_params* params, int n, const std::vector<const float*>& meshes);
    nf_status set_density(int r, int nx, int ny, int nz, const float* values);
    void release();
    nf_status cuda_fail(cudaError_t e, const char* where);

    // --- stages ------------------------------------------------------------
    nf_status setup();
    nf_status stream_dump(uint64_t k0, uint64_t n, float* host10);
    nf_status inject(size_t n, const float4* hpos, const float4* hdir, const uint64_t* hsidx);
    nf_status generate();
    nf_status rebuild_cells();
    nf_status contacts();
    nf_status solve();
    // Active-set CSR system of a graph (shared by the DC and AC solves).
    struct Asm {
        uint32_t na = 0, nnz = 0;
        bool chains = false;
        std::vector<uint32_t> habase;  // active base per realisation
    };
    nf_status assemble(uint32_t n, const std::vector<uint32_t>& off, uint32_t mc, uint32_t m, const uint32_t* eI,
                       const uint32_t* eJ, const double* eG, const double* eC, Asm* out);
    // Unscreened contact list for the statistics (the reference counts every
    // pair within the cutoff); *recomputed tells whether the handle's list
    // was replaced.
    nf_status unscreened_contacts(bool* recomputed);
    nf_status stat_nematic(const double axis[3], double* S);
    nf_status stat_phitheta(int bins_phi, int bins_theta, uint64_t* hist);
    nf_status stat_pairs(int bins, uint64_t* hist, uint32_t* per_rod, size_t capacity, nf_pair_stats* out);
    // Dead-end pruning (the reference's reduce): keep the min_cont-core of the
    // unscreened contact graph, electrodes kept.
    nf_status prune(int min_cont, nf_reduce_stats* out);
    // Stable compaction of rods [0, n) of a single realisation to those with
    // keep[i] != 0 (stream order kept), then a rebuild of the cell lists.
    nf_status compact_rods(const uint32_t* keep, uint32_t n, uint32_t left);
    // Adaptive generation: whether it is on, the law grid set-up (global law
    // in every cell), the refit + thin-out at an epoch boundary, and the
    // clusterisation of the round's kept candidates onto the n_old rods
    // present when the epoch began.
    bool adaptive() const;
    nf_status laws_reset();
    nf_status epoch_boundary(uint64_t epoch_done, uint32_t gained);
    nf_status epoch_boundary_tn(uint64_t epoch_done, uint32_t n);
    nf_status clusterize(uint64_t slots, const uint32_t* ntot, uint32_t n_old);
    // adds the snaps of the round's candidates with stream index < limit
    nf_status count_snaps(uint64_t slots, const uint32_t* ntot, uint64_t limit);
    nf_status orientation_laws(size_t cap, int32_t ext[3], float* axis, float* kappa, size_t* cells);
    // AC admittance spectrum of the handle's network (net == nullptr) or of a
    // host-given network.
    nf_status ac_spectrum(const nf_ac_net* net, const nf_ac_params& p, const double* freq, size_t nfreq,
                          nf_ac_point* out, nf_ac_stats* stats);
    // Edges [0, mc) are general; edges [mc, m) are chain links joining node i
    // to node i + 1 of the same rod (rod segments of the internal network).
    nf_status solve_graph(uint32_t n, const std::vector<uint32_t>& off, const std::vector<uint32_t>& nodes, uint32_t mc,
                          uint32_t m, const uint32_t* eI, const uint32_t* eJ, const double* eG);
    // Intra-rod resistor network (nodes = contact points, merged closer than a
    // radius; edges = contacts + rod segments); nf_solve uses it while int_valid.
    nf_status internal_network();
    bool int_valid = false;
    uint64_t int_nodes = 0, int_edges = 0, int_segs = 0, int_full = 0;
    std::vector<uint32_t> int_off, int_count;     // per realisation node ranges
    DBuf<uint32_t> inrod, ieI, ieJ, ivals, ivals2, inew, igid, islot;
    DBuf<double> int_t, ieG, iseg_l;
    DBuf<unsigned long long> ikeys, ikeys2;
    nf_status adjoint(int r, float* dG_dend, size_t cap, double* dlam, double* dg0);

    // helpers
    nf_status scan_u32(const uint32_t* in, uint32_t* out, size_t n);
    // Work list of (probe chunk, offset, target segment) items; the item
    // count lands in ioff[ncell * 27] and its maximum over calls in ctr[C_ITEMS].
    // np / nt: probes and targets in all cells, for the first capacity guess.
    // ring: 0 all stencil rows, 1 the inner rows (|dy|, |dz| <= 1), 2 the others.
    nf_status build_items(const uint32_t* pstart, const uint32_t* tstart, int stage, uint64_t np, uint64_t nt,
                          int ring = 0);
    // Tube registrations: the placed rods (stage 0 generation, 1 contacts)
    // into trod_*, the round's candidates (all kept, or the survivors of the
    // old-rod test) into tcnd_*; then the work list of probes x targets.
    // room: leave room in each cell for the rods of later rounds (appended by
    // tube_append_rods, the generation's rounds)
    nf_status tube_register_rods(int stage, bool room = false);
    nf_status tube_append_rods();
    // extra (a device counter) is read back with the registration's total
    nf_status tube_register_cands(uint64_t slots, const uint32_t* ntot, bool alive_only,
                                  const unsigned long long* extra = nullptr, unsigned long long* extra_out = nullptr);
    // Work items of a tube sweep (probe entries at pstart, target entries at
    // tstart, per-cell counts when compacted); pack: small cells in packed
    // items (the generation's sweeps read both kinds).
    nf_status tube_items(const uint32_t* pstart, const uint32_t* tstart, const uint32_t* pcnt = nullptr,
                         const uint32_t* tcnt = nullptr, bool pack = false);
    // Compacts the candidate registration (tcnd_*) in place to the candidates
    // still alive; per-cell lengths in tcnd_cnt.
    nf_status tube_compact_cands();
    // Registers objects [0, n) of any source (stage-1 periodicity) into tcnd_*.
    template <class Src>
    nf_status tube_register_objects(uint32_t n, Src src);
    const uint32_t* titem_count() const { return tioff.p + tit_nseg; }
    // Pinned host block for the per-round read-backs.
    uint8_t* hpin = nullptr;
    size_t hpin_cap = 0;
    nf_status ensure_pinned(size_t bytes);
    // Device address of the item count of the last build_items (read it after
    // that call: build_items may reallocate ioff).
    const uint32_t* item_count() const { return ioff.p + (size_t)ncell * kRows; }
    // Persistent grid of a pair kernel: as many kTPB-thread blocks as fit on
    // the device at once.
    template <class K>
    unsigned persistent_grid(K kernel) const {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kTPB, 0) != cudaSuccess || nb < 1) nb = 1;
        return (unsigned)(nsm * nb);
    }
    uint64_t total_rods() const;
};

// Count, scan, fill.
// grow (per realisation, on the device): leave room in each cell for that
// much growth (k_treg_room), the free slots marked kTubeRoom; the per-cell
// counts are then in cur. extra: a device counter read back with the total.
template <class Src>
inline nf_status tube_register(Engine& E, uint32_t n, const uint32_t* ntot, int stage, Src src, DBuf<uint32_t>& start,
                               DBuf<uint32_t>& cur, DBuf<uint32_t>& ent, DBuf<float4>& epos, DBuf<float4>& edir,
                               const float* grow = nullptr, const unsigned long long* extra = nullptr,
                               unsigned long long* extra_out = nullptr) {
    const uint32_t nc = E.ntcell;
    cudaStream_t st = E.st;
#define NF_CKT(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) return E.cuda_fail(e_, #x); } while (0)
    NF_CKT(start.ensure(nc + 1));
    NF_CKT(cur.ensure(nc + 1));
    NF_CKT(cudaMemsetAsync(cur.p, 0, sizeof(uint32_t) * (nc + 1), st));
    if (n) {
        auto kcount = k_treg<Src, 0>;
        NF_LAUNCH(kcount, (unsigned)((n + kRegTPB - 1) / kRegTPB), kRegTPB, 0, st)(
            n, ntot, E.dreal.p, stage, src, cur.p, nullptr, nullptr, nullptr, nullptr, 0u, nullptr);
        NF_CKT(cudaGetLastError());
    }
    if (grow && nc) {
        NF_LAUNCH(k_treg_room, (nc + 255) / 256, 256, 0, st)(nc, cur.p, E.toffs.p, E.R, grow);
        NF_CKT(cudaGetLastError());
    }
    nf_status s = E.scan_u32(cur.p, start.p, nc + 1);
    if (s != NF_OK) return s;
    // entries (with their objects' geometry, 36 B each) sized by the count:
    // one 4-byte read-back; an entry beyond the buffers would be counted in
    // C_TUBE_OVF, which fails the stage. The fill writes the 4-byte entries
    // alone (scattered); a second pass adds the geometry in entry order.
    s = E.ensure_pinned(16);
    if (s != NF_OK) return s;
    uint32_t* h = reinterpret_cast<uint32_t*>(E.hpin);
    unsigned long long* hx = reinterpret_cast<unsigned long long*>(E.hpin) + 1;
    NF_CKT(cudaMemcpyAsync(h, start.p + nc, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (extra) NF_CKT(cudaMemcpyAsync(hx, extra, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    NF_CKT(cudaStreamSynchronize(st));
    const size_t total = *h;
    if (extra && extra_out) *extra_out = *hx;
    (&start == &E.trod_start ? E.trod_total : E.tcnd_total) = total;
    NF_CKT(ent.ensure(total + 1));
    NF_CKT(epos.ensure(total + 1));
    NF_CKT(edir.ensure(total + 1));
    NF_CKT(cudaMemsetAsync(cur.p, 0, sizeof(uint32_t) * (nc + 1), st));
    if (grow) NF_CKT(cudaMemsetAsync(ent.p, 0xff, sizeof(uint32_t) * total, st));  // every slot kTubeRoom
    if (n) {
        auto kfill = k_treg<Src, 1>;
        NF_LAUNCH(kfill, (unsigned)((n + kRegTPB - 1) / kRegTPB), kRegTPB, 0, st)(
            n, ntot, E.dreal.p, stage, src, cur.p, start.p, ent.p, nullptr, nullptr,
            (uint32_t)std::min(ent.cap, std::min(epos.cap, edir.cap)), E.ctr.p + C_TUBE_OVF);
        NF_CKT(cudaGetLastError());
        if (total) {
            auto kgeom = k_treg_geom<Src>;
            NF_LAUNCH(kgeom, (unsigned)std::min<size_t>((total + 255) / 256, (size_t)E.nsm * 32), 256, 0, st)(
                (uint32_t)total, ent.p, epos.p, edir.p, src);
            NF_CKT(cudaGetLastError());
        }
    }
#undef NF_CKT
    return NF_OK;
}

template <class Src>
nf_status Engine::tube_register_objects(uint32_t n, Src src) {
    return tube_register(*this, n, nullptr, 1, src, tcnd_start, tcnd_cur, tcnd_ent, tcnd_pos, tcnd_dir);
}

// Derived realisation descriptor (identical arithmetic to the oracle).
Real make_real(const nf_params& p, const float* dmesh, int mn[3], double reach);
// Constants (c1, c2, zmax) of tn_angle for scale s on +- w (ref: the
// reference's sym_truncNormal form).
void tn_consts(float s, double w, int ref, double* c1, double* c2, double* zmax);
double stage_reach(const nf_params& p);
int64_t target_count(const nf_params& p);

}  // namespace nf
