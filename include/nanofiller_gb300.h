/*
 * nanofiller_gb300.h -- C ABI of the GB300-native NanoFiller hot path.
 *
 * The path: Monte Carlo rod candidates drawn from a density and an orientation
 * profile -> cell-list hard-core rejection with sequential-insertion semantics
 * -> tunnelling-contact extraction (count/record, screening, electrode roles)
 * -> conductance-network solve -> adjoint of the effective conductance.
 *
 * Conventions (all entry points):
 *   - every call returns nf_status; nothing prints, nothing exits;
 *   - lengths are in micrometres and angles in radians, like the reference's
 *     simPrms (src/simPrms.cpp:22-117);
 *   - host arrays are caller-owned; sizes are in elements;
 *   - one handle per host thread; a handle owns its device memory and runs on
 *     the stream given to nf_set_stream (default: the legacy stream);
 *   - no global device state: parameters travel in kernel arguments.
 *
 * Each declaration names the reference interface it replaces (file:line in
 * pyrlinum/NanoFiller).
 */
#ifndef NANOFILLER_GB300_H
#define NANOFILLER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NF_ABI_VERSION 1

/* Electrode pseudo-rod ids in contact lists (inc/definitions.h:18-20). */
#define NF_SRC_ELEC 0xFFFFFFFFu
#define NF_SNK_ELEC 0xFFFFFFFEu

typedef enum nf_status {
    NF_OK = 0,
    NF_ERR_PARAM = 1,         /* invalid parameter, size or pointer */
    NF_ERR_CUDA = 2,          /* CUDA runtime error (text in nf_last_error) */
    NF_ERR_NO_DEVICE = 3,     /* no CUDA device visible */
    NF_ERR_ALLOC = 4,         /* device or host allocation failed */
    NF_ERR_CAPACITY = 5,      /* caller buffer too small; ->count holds the need */
    NF_ERR_OVERFLOW = 6,      /* a fixed-capacity internal list overflowed */
    NF_ERR_NOT_CONVERGED = 7, /* the network solve missed its tolerance */
    NF_ERR_IO = 8,            /* file could not be opened or written */
    NF_ERR_FORMAT = 9,        /* malformed or truncated input file */
    NF_ERR_STATE = 10,        /* call out of order (e.g. contacts before rods) */
    NF_ERR_UNSUPPORTED = 11,  /* parsed reference option this path does not run */
    NF_ERR_TIMEOUT = 12       /* a bounded device-side wait gave up */
} nf_status;

enum { NF_ORIENT_ISOTROPIC = 0, NF_ORIENT_VMF = 1 };
enum { NF_SIZE_CONST = 0, NF_SIZE_LOGNORMAL = 1, NF_SIZE_UNIFORM = 2 };

/*
 * Parameters. The first block mirrors the reference keyword surface
 * (inc/parameter_input.h:8-68, parsed in src/simPrms.cpp:212-327; defaults
 * src/simPrms.cpp:22-117). The second block holds the project keys that the
 * reference has no keyword for (seeded stream, size and orientation laws,
 * tunnelling law, solver).
 */
typedef struct nf_params {
    /* --- reference keywords --- */
    float vf;               /* VOLUME_PERCENT / 100                          */
    float vf_precision;     /* VOL_FRAC_PRECISION (parsed; stop is exact)    */
    float box[3];           /* physDim: SPAT_DISTR_FILE NONE Lx Ly Lz        */
    int32_t mesh_ext[3];    /* SPAT_DISTR_FILE NONE ... nx ny nz             */
    char density_file[256]; /* SPAT_DISTR_FILE <file> (read_density format)  */
    float pref_ort[2];      /* PREF_ORT_PHI, PREF_ORT_THETA (rad)            */
    float theta_med;        /* DEF_THETA_MED (rad)                           */
    float theta_dev;        /* DEF_THETA_DEV (rad, <=0: cos theta uniform);
                               > 0: theta truncated normal about theta_med,
                               measured from the preferred axis            */
    float phi_med;          /* DEF_PHI_MED (rad)                             */
    float phi_dev;          /* DEF_PHI_DEV (rad, <=0: phi uniform); > 0: phi
                               truncated normal about phi_med (genCosine,
                               inc/cuda_CNTgenerate.h:262-270)             */
    float l;                /* INC_LEN_MED: rod length (median if lognormal) */
    float a;                /* INC_RAD_MED: rod radius                       */
    float l_dev;            /* INC_LEN_DEV (parsed)                          */
    float a_dev;            /* INC_RAD_DEV (parsed)                          */
    float sep;              /* INC_SEPARATION: hard-core gap                 */
    float sc_frac;          /* INC_SOFTCORE: hard-core radius fraction       */
    float tol;              /* TOL: geometric epsilon (1e-6)                 */
    float stat_dist_lim;    /* STAT_DIST_LIM: tunnelling cutoff              */
    int32_t wrt_bin;        /* WRT_BIN                                       */
    int32_t self_align_step;/* SELF_ALLIGN_STEP: law refit period in epochs  */
    int32_t clust_flag;     /* CLUST_FLAG: snap candidates to older rods     */
    int32_t reduce_flag;    /* REDUCE_FLAG: thin out after each refit        */
    /* --- project keys --- */
    uint64_t seed;          /* SEED: Philox4x32-10 key                       */
    uint64_t n_candidates;  /* CANDIDATES: stream budget                     */
    int64_t n_target;       /* TARGET_COUNT: 0 -> ceil(vf V / (pi a^2 l))    */
    int32_t gen_periodic;   /* PERIODIC: bitmask x=1 y=2 z=4                 */
    int32_t field_dir;      /* FIELD_DIR: electrode axis 1,2,4 (0: none)     */
    int32_t orient_mode;    /* ORIENT: NF_ORIENT_*                           */
    float vmf_kappa;        /* VMF_KAPPA                                     */
    int32_t len_mode;       /* LEN_LAW: NF_SIZE_CONST / NF_SIZE_LOGNORMAL    */
    float len_sigma_ln;     /* LEN_SIGMA_LN                                  */
    float len_min, len_max; /* LEN_CLIP lo hi                                */
    int32_t rad_mode;       /* RAD_LAW: NF_SIZE_CONST / NF_SIZE_UNIFORM      */
    float rad_min, rad_max; /* RAD_RANGE lo hi                               */
    float density_default;  /* DENSITY_DEFAULT: rho when no mesh (1.0)       */
    float cell_edge;        /* CELL_EDGE: 0 -> smallest legal edge           */
    double G0;              /* TUNNEL_G0 (S)                                 */
    double lambda;          /* TUNNEL_LAMBDA (um)                            */
    double d_c;             /* TUNNEL_DC (um): gap floor and law offset      */
    int32_t ref_parallel_typo; /* REF_PARALLEL_TYPO: hard-core parallel branch as in
                                  inc/intersection_dev.h:51                 */
    int32_t screening;      /* SCREENING: drop contacts crossed by a rod     */
    int32_t round_candidates; /* ROUND_CANDIDATES: candidates per round; 0 -> adaptive */
    int32_t solve_max_iter; /* SOLVE_MAX_ITER (inner FP32 CG iterations)     */
    double solve_tol;       /* SOLVE_TOL: FP64 relative residual             */
    /* --- tuning: speed only, results never depend on these --- */
    int32_t stencil_radius; /* STENCIL_RADIUS: cells of edge >= reach / r and a
                               (2r+1)^3 stencil; 0 -> 2 where the box allows  */
    float round_overshoot;  /* ROUND_OVERSHOOT: candidates drawn per round over
                               the expected need; 0 -> 1.5                    */
    double two_phase_work;  /* TWO_PHASE_WORK: candidates x rods of a round
                               above which the old-rod test runs in phases
                               (centre stencil row, the four rows beside it,
                               the four inner corner rows, outer rows;
                               survivors packed between them);
                               0 -> 1e10, < 0 -> never                      */
    /* --- intra-rod resistor network (stat_conduct ... internal) --- */
    double rod_sigma;       /* ROD_CONDUCTIVITY (S/um): a rod segment between
                               contact points conducts rod_sigma pi a / L with
                               L = dt / a (tools/kirchhoff/kirchhoff.py:90-95,
                               s0 = 6.7e7 S/m = 67 S/um, the default)       */
    /* --- electrodes --- */
    int32_t elec_buffer;    /* ELEC_BUFFER: 0 (default) electrodes are the two
                               planes of the field axis; 1 the reference's
                               `expand` buffer layers (src/simPrms.cpp:744-852):
                               periodic images of the rods beyond each face,
                               every contact with an image below the box is a
                               source contact and above it a sink contact
                               (get_elec_dmnID, inc/conductivity.h:71-90), one
                               per image rod                                 */
    int32_t ref_trunc_normal; /* TRUNC_NORMAL_REF: 1 draws DEF_THETA_DEV / DEF_PHI_DEV
                               angles by the reference's own formula a + 2 s
                               sqrt2 erfinv(Fa (1 - 2u)), Fa = erf(-w/s/sqrt2)/2
                               (sym_truncNormal, inc/cuda_CNTgenerate.h:271-275:
                               not a normal law); 0 (default) the exact normal
                               of deviation s truncated to a +- w (w = pi/2 for
                               theta, pi for phi)                            */
    /* --- adaptive generation: self-alignment, thin-out, clusterisation ---
     * The reference refits per-cell orientation laws every SELF_ALLIGN_STEP
     * rounds or when a round gained fewer than 1 % of the rods still missing
     * (src/cudaMain.cu:122-132), deletes rods that the new laws make unlikely
     * when REDUCE_FLAG is set (cudaThinOUT, src/cudaMain.cu:354-396) and, with
     * CLUST_FLAG, snaps each new candidate parallel to a nearby older rod
     * (cuda_Clusterize2Old, inc/cuda_Clusterize.h:14-100). Here the three act
     * at fixed epochs of the candidate stream (rounds are not part of the
     * result): self_align_step s > 0 refits after epoch e > 0 when e % s == 0
     * or the epoch gained fewer than (target - count) / 100 rods; reduce_flag
     * thins after each refit; clust_flag snaps the candidates of an epoch to
     * the rods present when it starts.                                      */
    float clust_dist;       /* CLUST_DIST_LIM (um): snap when the rods' closest
                               points are at most this far apart (0.015)   */
    float clust_angl;       /* CLUST_ANGL_LIM (rad): and their axes at most
                               this angle apart (pi / 12)                  */
    float align_cell;       /* ALIGN_CELL (um): edge of the orientation-law
                               cells; 0 -> the rod length INC_LEN_MED      */
    int32_t align_min;      /* ALIGN_MIN_RODS: rods a cell needs for a refit
                               (4); cells with fewer keep their law        */
    int64_t epoch_candidates; /* EPOCH_CANDIDATES: candidates per epoch;
                               0 -> max(1024, target count)                */
    int32_t solve_method;   /* SOLVE_METHOD: 0 auto (direct when the network's
                               band after reverse Cuthill-McKee is narrow:
                               block cyclic reduction up to 32, banded LDL^T
                               up to 512), 1 direct (the same, an error when
                               the band is wider), 2 iterative (PCG),
                               3 banded LDL^T                               */
    float tube_load;        /* TUBE_LOAD (tuning, speed only): the pair sweeps
                               register every rod in each cell of a fine grid
                               that its axis segment, dilated by half the
                               widest pair threshold, touches, and test the
                               pairs that share a cell; the cell edge is chosen
                               for about this many registrations per cell
                               (0 -> 64); < 0 -> the cell-stencil sweeps     */
    int32_t align_law;      /* ALIGN_LAW: the law a self-alignment refit gives
                               a cell. 0 (default) a von Mises-Fisher law
                               about the principal axis of the cell's
                               orientation tensor. 1 the reference's law
                               (crossMtxBuild / resetOrt / resetAvgVec,
                               inc/allignment_fit.h:154-458): preferred axis
                               = the eigenvector of the largest eigenvalue
                               when the two smaller ones are within 10 %,
                               else of the smallest; truncated-normal theta /
                               phi about the mean direction of the cell's
                               rods (when its norm per rod exceeds 0.5) with
                               their mean squared deviations as the scales,
                               drawn as DEF_THETA_DEV / DEF_PHI_DEV select
                               and rotated by the preferred axis; thin-out
                               by the reference's Gaussian likelihood        */
    int32_t autotune;       /* AUTOTUNE (tuning, speed only): 1 -> nf_batch_run
                               first runs nf_autotune on its batch (nine
                               more generations) and then contacts and
                               solves under the settings chosen; 0 (default)
                               the settings given                          */
} nf_params;

/* Rods, structure of arrays, caller-owned host buffers. Any array may be NULL. */
typedef struct nf_rods {
    size_t capacity;        /* in: rods the arrays hold                    */
    size_t count;           /* out: rods written (or needed on CAPACITY)   */
    float *x, *y, *z;       /* centre                                      */
    float *cx, *cy, *cz;    /* unit axis                                   */
    float *l, *a;           /* length, radius                              */
    uint64_t *stream_index; /* candidate index k that produced the rod     */
    uint32_t *cell;         /* global cell id (the reference's field k)    */
} nf_rods;

/* Contacts, sorted by (I, J). Electrode contacts carry J = NF_SRC_ELEC/NF_SNK_ELEC. */
typedef struct nf_contact_list {
    size_t capacity;
    size_t count;
    uint32_t *I, *J;        /* rod ids (acceptance order), I < J           */
    float *tI, *tJ;         /* clamped axis parameters of the contact pts  */
    double *D;              /* axis distance at (tI,tJ); gap = D - aI - aJ */
    double *G;              /* edge conductance (S)                        */
    double *S;              /* contact area estimate (um^2)                */
    int8_t *image;          /* 3 per contact: periodic image of J          */
} nf_contact_list;

typedef struct nf_gen_stats {
    uint64_t candidates_drawn;  /* stream indices consumed                 */
    uint64_t density_accepted;  /* candidates passing u < rho(x)           */
    uint64_t accepted;          /* rods                                    */
    uint64_t target;            /* rods asked for                          */
    uint64_t pair_tests;        /* FP32 filter evaluations                 */
    uint64_t exact_evals;       /* FP64 evaluations of the reference test  */
    uint64_t fp32_would_flip;   /* of those, decisions pure FP32 gets wrong*/
    int32_t rounds;
    int32_t target_reached;
    double ms;
    /* work of the two pair sweeps (candidates vs rods, vs earlier candidates) */
    uint64_t work_items;        /* (probe chunk, stencil row, segment) items  */
    uint64_t target_tiles;      /* 32-target tiles staged                    */
    uint64_t marked_pairs;      /* pairs passing the marking pre-tests (line
                                   bound, then capsule; on the stencil sweeps
                                   the conflict sweep marks by capsule only)  */
    uint64_t line_pairs;        /* of those, kept by the hand-out (relative
                                   image in range; on the stencil sweeps also
                                   its line bound)                            */
    /* adaptive generation (zero when it is off) */
    uint64_t epochs;            /* epochs of the candidate stream begun      */
    uint64_t refits;            /* orientation-law refits                     */
    uint64_t thinned;           /* rods removed by thin-out                   */
    uint64_t snapped;           /* snaps of candidates to older rods          */
    int32_t tube_grid;          /* 1: the pair sweeps ran on the tube grid    */
    int32_t redone_rounds;      /* rounds run again after a work list, FP64
                                   queue or conflict list overflowed (their
                                   buffers grow; results are unchanged)       */
} nf_gen_stats;

typedef struct nf_contact_stats {
    uint64_t contacts;          /* rod-rod contacts after screening        */
    uint64_t screened;          /* contacts dropped by screening           */
    uint64_t n_source, n_sink;  /* electrode contacts                      */
    uint64_t pair_tests, exact_evals, fp32_would_flip;
    double ms;
} nf_contact_stats;

typedef struct nf_solve_stats {
    double G_eff;               /* effective conductance (S)               */
    double residual;            /* final ||b - K v|| / ||b|| in FP64       */
    int32_t outer_iters;        /* FP64 refinement steps                   */
    int32_t inner_iters;        /* FP32 CG iterations, all steps           */
    int64_t n_nodes;            /* rods, or nodes of the internal network  */
    int64_t n_active;           /* unknowns: rods linked to both electrodes*/
    int32_t percolating;        /* a path joins source and sink            */
    double ms;
    int32_t direct;             /* 2: block cyclic reduction, 1: banded
                                   LDL^T (outer_iters = refinement steps,
                                   inner_iters = 0); 0: PCG                 */
    uint32_t bandwidth;         /* widest band after reordering (direct)    */
} nf_solve_stats;

typedef struct nf_batch_result {
    uint64_t accepted;
    uint64_t contacts;
    double G_eff;
    double residual;
    int32_t percolating;
    int32_t status;             /* nf_status of this realisation           */
} nf_batch_result;

typedef struct nf_batch_stats {
    int32_t n;
    int32_t rounds;
    uint64_t rods, contacts;
    double ms;
} nf_batch_stats;

typedef struct nf_handle nf_handle;

/* ---- library ---------------------------------------------------------- */
int nf_abi_version(void);
/* Human-readable name of a status code (static string). */
const char *nf_status_string(nf_status s);

/* ---- parameters (src/simPrms.cpp:22-117, :212-327) ---------------------- */
/* Fill with the reference defaults plus project defaults. */
nf_status nf_params_default(nf_params *p);
/* Parse a reference keyword file (inc/parameter_input.h:8-68) plus project
 * keys; unknown keys are counted in *n_unknown (may be NULL), as the
 * reference warns and continues (src/simPrms.cpp:317-319). */
nf_status nf_params_from_file(const char *path, nf_params *p, int *n_unknown);
/* Target count N = ceil(vf V / (pi a^2 l)) (src/simPrms.cpp:987-1002). */
nf_status nf_target_count(const nf_params *p, int64_t *n);

/* ---- handle ------------------------------------------------------------ */
/* Replaces the simPrms object + device set-up (src/simPrms.cpp:393-502,
 * src/cudaMain.cu:61-90). */
nf_status nf_create(const nf_params *p, nf_handle **out);
nf_status nf_destroy(nf_handle *h);
/* cudaStream_t passed as void*; NULL is the legacy stream. */
nf_status nf_set_stream(nf_handle *h, void *stream);
/* Last error text of this handle. */
nf_status nf_last_error(const nf_handle *h, char *buf, size_t n);

/* ---- inputs ------------------------------------------------------------ */
/* Density mesh, read_density order values[i*ny*nz + j*nz + k]
 * (src/IO.cpp:11-36; uploaded like density2Tex, inc/den2tex.h:5-53). */
nf_status nf_load_density(nf_handle *h, int nx, int ny, int nz,
                          const float *values);
/* Read a read_density file into host memory (header then values). */
nf_status nf_read_density_file(const char *path, int ext[3], float dim[3],
                               float *values, size_t capacity);

/* ---- generation (src/cudaMain.cu:61-161, :219-351) ---------------------- */
/* Draws the seeded stream until the target count or the budget is reached.
 * Accepted set == sequential insertion in stream order. */
nf_status nf_generate(nf_handle *h, nf_gen_stats *stats);
/* Candidate stream itself (for checking): candidates [k0, k0+n), all fields,
 * with the von Neumann variate in u and rho(x) in rho. */
nf_status nf_stream_candidates(nf_handle *h, uint64_t k0, uint64_t n,
                               float *x, float *y, float *z, float *cx,
                               float *cy, float *cz, float *l, float *a,
                               float *u, float *rho);
/* Same candidates as nf_stream_candidates, through a call that allocates
 * nothing (no reference counterpart). For callers that may not allocate
 * while they run: a host framework that has handed all free device memory
 * to its own caching allocator, or a checker that samples the stream while
 * nf_generate runs on another stream of the same device and must not stall
 * it (cudaFree synchronises the whole device). The staging buffer is a
 * fixed device array of NF_NOALLOC_MAX_CANDIDATES x 10 floats (2.5 MiB)
 * inside the library; n above NF_NOALLOC_MAX_CANDIDATES returns
 * NF_ERR_CAPACITY. Nothing in that array needs to start at zero: each call
 * writes every value it copies out. Every call looks up the array's device
 * address on the handle's device (cudaGetSymbolAddress; the first call on a
 * device may load the library's device code: make it before any stream
 * capture begins), so no address outlives a device reset. Calls on the same
 * device share the array, so two calls in flight
 * at once (different streams or host threads) race: serialise them. A handle
 * with a density mesh must have uploaded it first (nf_generate or
 * nf_stream_candidates after nf_create / nf_load_density), else
 * NF_ERR_STATE; the current device must be the handle's. */
#define NF_NOALLOC_MAX_CANDIDATES 65536u
nf_status nf_stream_candidates_noalloc(nf_handle *h, uint64_t k0, uint64_t n,
                                       float *x, float *y, float *z, float *cx,
                                       float *cy, float *cz, float *l, float *a,
                                       float *u, float *rho);
/* Copy the accepted rods out (simPrms::asmbl_cnt_data, src/simPrms.cpp:329-391). */
nf_status nf_get_rods(nf_handle *h, nf_rods *out);
/* Replace the rod set (inject, e.g. from output.bin; stream_index may be NULL). */
nf_status nf_set_rods(nf_handle *h, const nf_rods *in);

/* ---- contacts (src/conductivity.cu:140-226, src/get_contact_arrays.cu:12-140,
 *      src/check_screened_Interactions.cu:12-70, src/get_contact_data.cu:28-230) */
nf_status nf_contacts(nf_handle *h, nf_contact_stats *stats);
/* Rod-rod contacts first, then sink, then source (save_coo order). */
nf_status nf_get_contacts(nf_handle *h, nf_contact_list *out);

/* ---- network solve (tools/kirchhoff/kirchhoff.py:211-269,
 *      tools/kirchhoff/lib/solver.cpp:185-269) --------------------------- */
nf_status nf_solve(nf_handle *h, nf_solve_stats *stats);
/* Node voltages (rods; 0 for rods outside the source-sink network). */
nf_status nf_get_voltages(nf_handle *h, double *v, size_t capacity);

/* ---- intra-rod resistor network (stat_conduct dir internal:
 *      src/conductivity.cu:228-416,639-836, src/adjacency_graph.cu:57-219,
 *      tools/kirchhoff/kirchhoff.py:90-95) ------------------------------- */
/* Builds the node network from the current contacts: every contact end is a
 * node (rod, t); a node no more than one radius past its predecessor on the
 * rod merges into it (mean t); consecutive nodes of a rod are joined by a rod
 * segment of conductance rod_sigma pi a / L, L = dt / a. Until the next
 * nf_contacts or nf_generate, nf_solve solves this network (nf_get_voltages
 * then returns node voltages) and nf_adjoint reports NF_ERR_UNSUPPORTED. */
typedef struct nf_internal_stats {
    uint64_t contact_ends;      /* nodes before merging                       */
    uint64_t nodes;             /* nodes after merging                        */
    uint64_t segments;          /* rod segments                               */
} nf_internal_stats;
nf_status nf_internal_network(nf_handle *h, nf_internal_stats *stats);
/* The node network: nodes ordered by (rod, t); segments (i, j = i + 1, L, G);
 * every contact's two nodes in nf_get_contacts order (j keeps the electrode
 * id of electrode contacts). Any array may be NULL; counts are always set. */
typedef struct nf_internal_net {
    size_t capacity;        /* in: entries every non-NULL array holds        */
    size_t n_nodes, n_segments, n_edges;
    uint32_t *node_rod;
    double *node_t;
    uint32_t *seg_i, *seg_j;
    double *seg_l, *seg_g;
    uint32_t *edge_i, *edge_j;
} nf_internal_net;
nf_status nf_get_internal_network(nf_handle *h, nf_internal_net *out);
/* Nodes.tbl.dat, segment.LA.coo, internal.DS.coo, sink.DS.coo, source.DS.coo
 * in dir (save_coo layouts, src/conductivity.cu:881-930). */
nf_status nf_write_internal_coo(nf_handle *h, const char *dir);

/* ---- orientation law at run time ------------------------------------- */
/* The orientation keywords of simPrms (ORIENT, VMF_KAPPA, PREF_ORT_PHI,
 * PREF_ORT_THETA; src/simPrms.cpp:212-327) for the candidates drawn after
 * this call, in every realisation of the handle: NF_ORIENT_ISOTROPIC, or
 * NF_ORIENT_VMF with concentration kappa > 0 about the preferred axis
 * (pref_phi, pref_theta) in radians. Rods already accepted stay. */
nf_status nf_set_orientation(nf_handle *h, int32_t mode, float kappa, float pref_phi, float pref_theta);

/* Per-cell orientation laws of the adaptive generation (self_align_step > 0
 * or clust_flag), after nf_generate. ext[3] receives the law grid; for cell
 * i + ext[0] (j + ext[1] k), axis[3 cell..] the law's axis and kappa[cell]
 * its von Mises-Fisher concentration (0: isotropic). The reference keeps the
 * same per cell (d_prefOrt, d_thetaMed/Dev, d_phiMed/Dev; resetOrt and
 * resetAvgVec, inc/allignment_fit.h:214-458). NF_ERR_STATE when the handle
 * generates without adaptive laws; NF_ERR_CAPACITY (count in *cells) when
 * cap is too small. Either array may be NULL. */
nf_status nf_orientation_laws(nf_handle *h, size_t cap, int32_t ext[3], float *axis, float *kappa, size_t *cells);

/* ---- dead-end pruning: the `reduce` verb (src/NanoFiller.cpp:71-91) ---- */
/* Replaces the reference's reduce loop (reduce(), src/conductivity.cu:79-138;
 * contact_count_kernel_full / reductKernel, inc/conductKernels.h:39-162):
 * contacts within stat_dist_lim are counted per rod without screening
 * (electrode contacts count, electrodes are never removed), every rod with
 * fewer than min_contacts goes, and the count repeats until nothing goes.
 * The handle keeps the surviving rods in their order (stream indices kept);
 * contacts and solutions are dropped. */
typedef struct nf_reduce_stats {
    uint64_t rods_before;
    uint64_t rods_after;
    uint64_t contacts;      /* unscreened contacts of the first count */
    int32_t rounds;         /* passes that removed rods */
    int32_t min_contacts;
    double ms;
} nf_reduce_stats;

nf_status nf_reduce(nf_handle *h, int32_t min_contacts, nf_reduce_stats *stats);

/* ---- statistics and writers (src/NanoFiller.cpp:92-147) -------------- */
/* stat_nematic (get_nematic_order, src/statistics_collection.cu:589-638):
 * S = sum P2(c . axis) / N over the rods (unit axis; the verb uses z). */
nf_status nf_stat_nematic(nf_handle *h, const double axis[3], double *S);
/* stat_phitheta (collect_PhiTheta_distr, src/statistics_collection.cu:
 * 769-863): histogram of rod directions, bins_phi x bins_theta over
 * [0, pi] x [0, pi], phi fastest; the verb uses 32 x 32 and writes rho.dat. */
nf_status nf_stat_phitheta(nf_handle *h, int32_t bins_phi, int32_t bins_theta, uint64_t *hist);
/* stat_contacts and stat_mutangle (collect_CntctPerInc :463-586,
 * collect_1D_statDistr_weightedFloat :640-767): over the unscreened
 * rod-rod contacts within STAT_DIST_LIM, contacts per rod (both ends) and the
 * histogram of mutual angles acos|c_i . c_j| of the pairs whose closest
 * points are interior to both rods, bins of (pi + TOL) / 2 / bins; the verb
 * uses 32 bins and writes gamma.dat. If the handle's contacts are screened
 * ones, an unscreened sweep replaces them and they are dropped afterwards.
 * hist (bins) and per_rod (capacity >= rods) may be NULL. */
typedef struct nf_pair_stats {
    uint64_t rods;
    uint64_t pairs;          /* rod-rod contacts */
    uint64_t contacts_total; /* sum over rods of their contacts (2 x pairs) */
    uint64_t angle_pairs;    /* pairs in the mutual-angle histogram */
    uint32_t max_per_rod;
    uint32_t pad;
    double mean_per_rod;
} nf_pair_stats;
nf_status nf_stat_pairs(nf_handle *h, int32_t bins, uint64_t *hist, uint32_t *per_rod, size_t capacity,
                        nf_pair_stats *stats);
/* write_ort (write_CNT_ORTvtk, src/IO.cpp:77-97): rod directions as VTK points. */
nf_status nf_write_ort_vtk(nf_handle *h, const char *path);
/* write_lmp (write_CNTlmp, src/IO.cpp:99-146): LAMMPS data file of
 * ellipsoids (length l + 2a, width 2a, quaternion from x to the rod axis);
 * density per particle as the reference's simPrms density (4.579). */
nf_status nf_write_lmp(nf_handle *h, const char *path, double density);
/* The verbs' histogram files: rho.dat (write_Mathematica2Di, src/IO.cpp) and
 * gamma.dat (write_mat, src/IO.cpp). Host-only. */
nf_status nf_format_write_rho(const char *path, int32_t bins_phi, int32_t bins_theta, const uint64_t *hist);
nf_status nf_format_write_gamma(const char *path, int32_t bins, const uint64_t *hist);

/* ---- AC admittance spectrum (tools/kirchhoff/kirchhoff.py) ------------ */
/* The offline Kirchhoff tool's impedance sweep, restated: every edge gets the
 * scaled admittance Y = G + i (omega / omega0) C, with
 *   rod segment (L in radii, radius a):  G = sigma pi a / L * R0, C = 0
 *                                          (sigma = nf_params.rod_sigma)
 *   contact (axis distance D, area S):    d = max(D - 2 r_cnt, delta_min),
 *     S clamped to [pi r_cnt^2, 2 r_cnt l_cnt]; dropped unless d < delta_eff;
 *     G = (S / S_min) / (exp(B (d - delta_min)) d / delta_min) if d <= delta_tun
 *     else 0; C = (S / S_min) / (d / delta_min), 0 if below c_min
 * with A, B, R0 = A exp(B delta_min) delta_min / S_min, C0 = eps0 eps_r S_min /
 * delta_min and omega0 = 1 / (R0 C0) from the barrier phi (kirchhoff.py:
 * 55-116). Source at 1, sink at 0 (Norton form); I = sum over source
 * contacts of Y_src (1 - V), Z = R0 L_box / I (kirchhoff.py:211-286). Lengths
 * in um. One complex-symmetric solve per frequency, all frequencies of a call
 * in one launch (a CTA each). */
typedef struct nf_ac_params {
    double r_cnt;       /* um: radius of the gap correction and of S_min (4.75e-3) */
    double l_cnt;       /* um: S_max = 2 r_cnt l_cnt (1.5) */
    double phi_ev;      /* barrier height, eV (3.5) */
    double eps_r;       /* relative permittivity of the matrix (2.9) */
    double delta_min;   /* um: gap floor (0.34e-3) */
    double delta_tun;   /* um: tunnelling range (1.1e-3) */
    double delta_eff;   /* um: electrostatic range R_cut; farther contacts dropped */
    double c_min;       /* scaled capacitances below it are 0 (0.005) */
    double l_box;       /* um: impedance scale Z = R0 l_box / I */
    int32_t own_radii;  /* 0: gap D - 2 r_cnt for every contact (the tool);
                           1: D - a_I - a_J, electrode contacts D - a_I (the
                           handle's own network with plane electrodes) */
    int32_t method;     /* 0: banded LDL^T per frequency when the reordered
                           band is narrow enough, else COCG; 1: banded
                           (NF_ERR_PARAM if too wide); 2: COCG */
    double tol;         /* relative FP64 residual per frequency (1e-10) */
} nf_ac_params;

typedef struct nf_ac_point {
    double freq;        /* Hz */
    double i_re, i_im;  /* I in units of 1 / R0 */
    double z_re, z_im;  /* R0 l_box Re(1/I) and -R0 l_box Im(1/I), the
                           columns of impedance_rRC.<patch>.dat */
    double rms;         /* || K V - b ||_2 (the tool's RMS column) */
    double residual;    /* || K V - b || / || b ||; converged when <= tol */
    double i_err;       /* |V^T (b - K V)|: first-order error of I (K is
                           symmetric, so dI = b^T K^-1 r); the solve runs to
                           the FP64 rounding floor, so i_err / |I| says how
                           many digits of I are resolved */
    int32_t iters;      /* inner iterations */
    int32_t converged;
} nf_ac_point;

typedef struct nf_ac_stats {
    uint64_t n_nodes, n_active, n_contacts, n_kept, n_segments;
    double R0, C0, omega0;  /* ohm, F, rad/s */
    double ms;              /* device time of the call */
    uint32_t bandwidth;     /* of the active system after reverse Cuthill-McKee */
    int32_t direct;         /* 1: banded LDL^T per frequency; 0: COCG (bands too wide) */
} nf_ac_stats;

/* A network given on the host (the tool's input files): nodes 0..n_nodes-1,
 * segments (i, j = i + 1 of the same rod, L in radii, radius a in um),
 * contacts (i, j node or NF_SRC_ELEC / NF_SNK_ELEC, axis distance D in um,
 * area S in um^2). */
typedef struct nf_ac_net {
    uint64_t n_nodes;
    uint64_t n_segments;
    const uint32_t *seg_i, *seg_j;
    const double *seg_l, *seg_a;
    uint64_t n_contacts;
    const uint32_t *ct_i, *ct_j;
    const double *ct_d, *ct_s;
} nf_ac_net;

void nf_ac_params_default(nf_ac_params *p);
/* The tool's frequency grid (Hz): 10^(log_df x + logF_min), logF in [-2, 14],
 * split into n_patch patches of ceil(N / n_patch) points (kirchhoff.py:72-79,
 * 176). Returns the count; writes at most capacity values. */
size_t nf_ac_frequencies(double log_df, int n_patch, int patch_id, double *freq, size_t capacity);
/* net == NULL: the handle's own network (the intra-rod network after
 * nf_internal_network, else the rod-level contact network; one realisation).
 * Otherwise the given host network; h then only supplies the stream, the
 * device workspace and rod_sigma. Returns NF_ERR_NOT_CONVERGED if a
 * frequency missed tol (all points are still filled). */
nf_status nf_ac_spectrum(nf_handle *h, const nf_ac_net *net, const nf_ac_params *p, const double *freq,
                         size_t n_freq, nf_ac_point *out, nf_ac_stats *stats);

/* ---- adjoint (no reference counterpart) ------------------------------- */
/* dG_eff/d(endpoints) as N x 6 (e0.xyz, e1.xyz with e0/1 = r -/+ l/2 c),
 * dG_eff/dlambda and dG_eff/dG0, contact topology held fixed. */
nf_status nf_adjoint(nf_handle *h, float *dG_dend, size_t capacity,
                     double *dG_dlambda, double *dG_dG0);

/* ---- batched realisations (no reference counterpart; the reference runs
 *      one realisation per process, src/NanoFiller.cpp:37-162) ------------ */
/* One call: a batch handle is created, generated, contacted, solved and
 * destroyed; out[r] holds realisation r's result, stats->ms the device time
 * from the first generation launch to the end of the solve (tuning included
 * when params[0].autotune is 1: the tuner's settings then apply to every
 * realisation). */
nf_status nf_batch_run(const nf_params *params, int n, nf_batch_result *out,
                       nf_batch_stats *stats);
/* A handle holding n realisations side by side (own boxes, fractions,
 * seeds, density files): nf_generate, nf_contacts and nf_solve run all of
 * them in shared launches and may be called again (each call starts the
 * stage over); nf_set_stream and nf_set_kernel_timing apply as for one
 * realisation. nf_select(h, r) picks the realisation that nf_get_rods,
 * nf_get_contacts, nf_adjoint and the stats of nf_solve report (0 after
 * creation); calls that write files or statistics return NF_ERR_STATE on a
 * handle of more than one realisation. */
nf_status nf_create_batch(const nf_params *params, int n, nf_handle **out);
nf_status nf_select(nf_handle *h, int32_t r);
/* Per-realisation results of the last nf_solve of a batch handle (n must be
 * its realisation count). */
nf_status nf_batch_results(nf_handle *h, nf_batch_result *out, int32_t n);

/* ---- files ------------------------------------------------------------- */
/* VTK rods (src/IO.cpp:38-76). */
nf_status nf_write_vtk(nf_handle *h, const char *path);
/* output.bin state (src/stateSR.cpp:54-89 / :90-134). */
nf_status nf_write_state_bin(nf_handle *h, const char *path);
nf_status nf_read_state_bin(nf_handle *h, const char *path);
/* internal.srt.coo, sink.elec.coo, source.elec.coo in dir (src/conductivity.cu:838-879). */
nf_status nf_write_coo(nf_handle *h, const char *dir);

/* ---- autotuner (no reference counterpart) -------------------------------- */
/* Times full generations of the handle's realisations (one, or all of a
 * batch) under candidate values of the speed-only settings, one coordinate at
 * a time, each trial run twice and timed on the second, and keeps the fastest
 * in every realisation's parameters: on the tube grid (the default) the cell
 * edge through tube_load (32, 48, 64, 96, 128 but the value on entry) and
 * the candidates per round through round_overshoot (three of 1.25, 1.5, 2, 3
 * besides the value on entry); on the stencil
 * sweeps stencil_radius, round_overshoot and two_phase_work. The accepted
 * sets do not depend on them: the handle ends holding the rods nf_generate
 * gives. out may be NULL. */
typedef struct nf_tune_result {
    int32_t stencil_radius;
    float round_overshoot;
    double two_phase_work;
    double ms_first;        /* generation time with the settings on entry   */
    double ms_best;         /* with the settings chosen                     */
    int32_t trials;
    float tube_load;        /* chosen tube load (0: the default, 64)        */
} nf_tune_result;
nf_status nf_autotune(nf_handle *h, nf_tune_result *out);

/* ---- diagnostics (no reference counterpart; the reference prints timers,
 *      src/cudaMain.cu:147,157) ------------------------------------------ */
/* Kernel launches issued by this library in this process. */
uint64_t nf_kernel_launches(void);
/* Device and pinned host blocks this library requested in this process
 * (served by cudaMalloc, cudaMallocHost or its own block cache). */
uint64_t nf_allocations(void);
/* The library keeps the device blocks that destroyed handles and regrown
 * buffers give back, per device, and hands them to the next handle of the
 * process (at most a quarter of the device's memory, at most 64 GiB); this
 * call returns every cached block to the driver. (No reference counterpart.) */
nf_status nf_release_cached_memory(void);
/* Record CUDA events around the hot kernels on the handle's stream. */
nf_status nf_set_kernel_timing(nf_handle *h, int on);
/* Totals since timing was enabled for kernel "stream", "old_test",
 * "conflicts", "ct_pairs", "screen" or "cg": device ms, launches, and the
 * algorithmic bytes / flops those launches had to move / compute. */
nf_status nf_kernel_time(nf_handle *h, const char *kernel, double *ms,
                         uint64_t *launches, double *bytes, double *flops);

/* Host-only format writers/readers on caller arrays (no device needed). */
nf_status nf_format_write_vtk(const char *path, size_t n, const float *x,
                              const float *y, const float *z, const float *cx,
                              const float *cy, const float *cz, const float *l,
                              const float *a, const float *k);
/* orient.vtk: the directions as points (write_CNT_ORTvtk, src/IO.cpp:77-99). */
nf_status nf_format_write_ort_vtk(const char *path, size_t n, const float *cx,
                                  const float *cy, const float *cz);
/* output.lmp.data: LAMMPS ellipsoids (write_CNTlmp, src/IO.cpp:100-146). */
nf_status nf_format_write_lmp(const char *path, size_t n, const float *x,
                              const float *y, const float *z, const float *cx,
                              const float *cy, const float *cz, const float *l,
                              const float *a, const float box[3], double density);
typedef struct nf_state_header {
    float phys_dim[3];
    float edge[3];
    int32_t ext[3];
    float l, a;
    int32_t ttl;            /* slots (== rods after repack)                */
    int32_t num;            /* rods                                        */
    float tol;
} nf_state_header;
nf_status nf_format_write_state_bin(const char *path, const nf_state_header *hd,
                                    const int16_t *occ, const int32_t *addr,
                                    const float *planes /* 9 x ttl */);
/* Reads the header; occ/addr/planes may be NULL to query sizes first. */
nf_status nf_format_read_state_bin(const char *path, nf_state_header *hd,
                                   int16_t *occ, int32_t *addr, float *planes,
                                   size_t cells_cap, size_t planes_cap);

#ifdef __cplusplus
}
#endif
#endif /* NANOFILLER_GB300_H */
