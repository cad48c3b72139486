/*
 * nf_oracle.h -- CPU oracle for the NanoFiller hot path (TEST INFRASTRUCTURE).
 *
 * This library is the oracle, used only to check and to time a CPU baseline:
 * only the tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * load it. The product library never links it.
 *
 * It restates, in plain C++ evaluated in FP64 (or FP32 for pinning against the
 * reference's own source), the reference's algorithm for:
 *   - the hard-core predicate  cnt_intersec_shr      inc/intersection_dev.h:10-80
 *   - the contact routine      distance_cylinder_capped
 *                              inc/intersect/intersect_cylinder_capped.h:69-167
 *   - the screening body test  body_intersect_cylinder_capped  (same file :181-191)
 *   - the virtual inclusion    generate_virt_inclusions  inc/conductKernels.h:289-361
 *   - the contact-area estimate surf_to_cylinder_capped (same file :204-293)
 *   - the target count         simPrms::set_numCNT       src/simPrms.cpp:987-1002
 *   - the clusterisation snap  cuda_Clusterize2Old / cnt_minDist
 *                              inc/cuda_Clusterize.h:14-100, inc/intersection_dev.h:85-160
 *   - the Norton assembly and G_eff  tools/kirchhoff/kirchhoff.py:232-269
 * plus the project-defined seeded candidate stream (Philox4x32-10, Salmon et al.
 * 2011) and sequential insertion in stream order.
 */
#ifndef NF_ORACLE_H
#define NF_ORACLE_H
#include <stdint.h>
#include "../include/nanofiller_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nfo_rod { float x, y, z, cx, cy, cz, l, a; } nfo_rod;

/* Philox4x32-10 block. */
void nfo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Deterministic float math of the stream contract. */
void nfo_sincos_turns(float t, float *c, float *s);
double nfo_erf(double x);
double nfo_erfinv(double y, double zmax);
double nfo_log_d(double x);
double nfo_exp_d(double x);
float nfo_logf(float v);
float nfo_expf(float x);

/* Reference routine on one pair. kind 0: hard-core test (cnt_intersec_shr),
 * kind 1: contact routine (distance_cylinder_capped). B is shifted by shift[]
 * (its periodic image) before the test, as tarnsCNT does. use_double selects
 * FP64 or FP32 evaluation. out = {d, t0, t1, Dtt.x, Dtt.y, Dtt.z}.
 * thr_sep is `sep` (kind 0) or `separation` (kind 1); scf the soft-core fraction.
 * Returns the hit decision. */
int nfo_pair_eval(int use_double, int kind, const nfo_rod *A, const nfo_rod *B,
                  const double shift[3], double eps, double scf, double thr_sep,
                  int typo, double out[6]);

/* Screening body test of a real rod A against a virtual rod given in FP64
 * (centre, unit axis, length, radius). Returns 1 if the virtual rod is crossed. */
int nfo_screen_eval(const nfo_rod *A, const double vr[3], const double vc[3],
                    double vl, double va, const double shift[3], double eps);

/* Contact area (surf_to_cylinder_capped) in FP64. */
double nfo_contact_area(const nfo_rod *A, const nfo_rod *B, const double shift[3],
                        double Dtt_x, double t0u, double t1u, double rlim);

/* Brute force over all images: for each probe i, the first rod j (array order)
 * with sidx[j] < k[i] that the probe hits in the FP64 hard-core test of the
 * generation stage, or -1. For checking accepted / rejected decisions. */
int64_t nfo_first_hits(const nf_params *p, const nfo_rod *probes, const uint64_t *k, int64_t m,
                       const nfo_rod *rods, const uint64_t *sidx, int64_t n, int nthreads, int64_t *out);

/* Intra-rod resistor network from a contact list (I, J, tI, tJ; electrode
 * contacts carry J = NF_SRC_ELEC / NF_SNK_ELEC): merged nodes (rod, t),
 * segments between consecutive nodes of a rod (L = dt / a, conductance
 * rod_sigma pi a / L) and each contact's two node ids (edge_j keeps the
 * electrode id). Arrays sized cap (edge arrays m). counts = {nodes, segments,
 * nodes before merging}. Returns the node count, -2 when cap is too small. */
int64_t nfo_internal_network(const nf_params *p, const nfo_rod *rods, int64_t n_rods, int64_t m,
                             const uint32_t *I, const uint32_t *J, const double *tI, const double *tJ,
                             int64_t cap, uint32_t *node_rod, double *node_t, uint32_t *seg_i, uint32_t *seg_j,
                             double *seg_l, double *seg_g, uint32_t *edge_i, uint32_t *edge_j, int64_t counts[3]);

/* One clusterisation step of a candidate against an older rod shifted by
 * shift[] (its periodic image): centre test, axis angle <= clust_angl,
 * cnt_minDist <= clust_dist, then the move parallel to the older rod at
 * a + a' + sep from its axis. out = the candidate after the step; returns 1
 * when it moved. */
int nfo_clust_snap(const nf_params *p, const nfo_rod *cand, const nfo_rod *older, const float shift[3],
                   nfo_rod *out);

/* Orientation law of a cell from its tensor sums {n, xx, yy, zz, xy, xz, yz}
 * (each product c_i c_j rounded to 2^-40 units): law[0..8] rotation (column 2
 * the axis), law[9] kappa, law[10] exp(-2 kappa), law[11] sampling flags. */
int nfo_fit_law(const int64_t sums[7], int sample, float law[12]);
/* ALIGN_LAW 1: the reference's truncated-normal law of one cell from the
 * directions (n x 3) of its rods: law[14] (rotation, flags, medians), lawd[10]
 * (medians and scales, tn_angle constants). */
int nfo_tn_cell_law(const float* dirs, int64_t n, int ref, float law[14], double lawd[10]);

/* Candidate stream k0..k0+n-1: out[10*i + f], f = x y z cx cy cz l a u rho. */
int nfo_candidates(const nf_params *p, const float *mesh, int nx, int ny, int nz,
                   uint64_t k0, uint64_t n, float *out);

/* Sequential insertion in stream order. batch>1 tests batches in parallel and
 * resolves in-batch conflicts in index order (identical result).
 * With self_align_step > 0 or clust_flag, the adaptive generation: epochs of
 * epoch_candidates, per-cell orientation laws refit at epoch boundaries from
 * exact tensor sums (principal axis, von Mises-Fisher concentration matched
 * to the largest eigenvalue), thin-out after a refit (reduce_flag), and the
 * snap of each kept candidate to the older rods near it (clust_flag).
 * stats = {drawn, density_accepted, pair_evals, epochs, refits, thinned,
 * snapped}; laws_out (12 floats per law cell, if laws_cap allows) and
 * law_ext receive the final laws. Returns accepted count or <0. */
int64_t nfo_generate(const nf_params *p, const float *mesh, int nx, int ny, int nz,
                     int nthreads, int64_t batch, int brute_force, int64_t cap,
                     nfo_rod *rods, uint64_t *stream_index, uint64_t stats[7], float *laws_out,
                     int64_t laws_cap, int32_t law_ext[3]);

/* Contacts: rod-rod (sorted I,J,image; screened ones removed), then sink, then
 * source. counts = {internal, screened, sink, source}. Returns total or <0.
 * Arrays sized cap. Electrode ids as in nanofiller_gb300.h. */
int64_t nfo_contacts(const nf_params *p, const nfo_rod *rods, int64_t n, int nthreads,
                     int brute_force, int64_t cap, uint32_t *I, uint32_t *J,
                     double *tI, double *tJ, double *D, double *G, double *S,
                     int8_t *img, int64_t counts[4]);

/* Network solve by Jacobi-preconditioned CG in FP64 on the rods joined to both
 * electrodes. v (n) receives voltages (1 on components touching only the source,
 * 0 on other rods outside the network). info = {iters, n_active,
 * percolating, residual}. Returns G_eff. */
double nfo_solve(int64_t n_rods, int64_t n_contacts, const uint32_t *I,
                 const uint32_t *J, const double *G, double tol, int max_iter,
                 double *v, double info[4]);

/* Adjoint: dG/d(endpoints) N x 6, dG/dlambda, dG/dG0 (FP64). */
void nfo_adjoint(const nf_params *p, const nfo_rod *rods, int64_t n_rods,
                 int64_t n_contacts, const uint32_t *I, const uint32_t *J,
                 const double *tI, const double *tJ, const double *D,
                 const double *G, const int8_t *img, const double *v,
                 double *dG_dend, double *dG_dlambda, double *dG_dG0);

#ifdef __cplusplus
}
#endif
#endif
