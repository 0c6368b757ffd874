/*
 * exptool_gb300 — C ABI of the GB300 (sm_103a) basis-function-expansion path.
 *
 * Every entry point returns an int status (XT_OK = 0, negative on error) and
 * never throws across the ABI; xt_last_error() returns the message of the
 * last failure on the calling thread.  Particle arrays, coefficient arrays,
 * outputs and workspaces are DEVICE pointers owned by the caller; table
 * handles own their device copies of the basis tables.  `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Calls are asynchronous with
 * respect to the host unless stated otherwise.
 *
 * The reference interfaces each entry point replaces are cited as
 * exptool/<file>:<line> (exptool 0.4.0, pure Python/NumPy).
 */
#ifndef EXPTOOL_GB300_H
#define EXPTOOL_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XT_OK 0
#define XT_ERR_ARG (-1)     /* invalid argument / size mismatch          */
#define XT_ERR_CUDA (-2)    /* CUDA runtime error                        */
#define XT_ERR_OOM (-3)     /* device allocation failed                  */
#define XT_ERR_WORKSPACE (-4) /* workspace too small                     */
#define XT_ERR_DEVICE (-5)  /* a kernel reported an error flag           */

/* precision of the per-particle arithmetic */
#define XT_F64 0            /* plain FP64: the drop-in path              */
#define XT_F32 1            /* FP32 per-particle work, FP64 reductions   */

/* coordinate modes of evaluation inputs (a, b, c) */
#define XT_COORD_CART 0     /* x, y, z                                   */
#define XT_COORD_SPH 1      /* r, cos(theta), phi   (spherical basis)    */
#define XT_COORD_CYL 1      /* R, z, phi            (cylindrical basis)  */

/* spherical evaluation modes */
#define XT_SPH_ALL_EVAL_PARTICLES 0 /* spheresl.all_eval_particles  (spheresl.py:1240) */
#define XT_SPH_ALL_EVAL 1           /* spheresl.all_eval            (spheresl.py:987)  */
#define XT_SPH_FORCE_EVAL 2         /* spheresl.force_eval          (spheresl.py:1107) */

/* cylindrical evaluation modes */
#define XT_CYL_ACCUMULATED_EVAL_PARTICLES 0 /* eof.accumulated_eval_particles (eof.py:989) */
#define XT_CYL_FORCE_EVAL 1                 /* eof.force_eval                 (eof.py:756) */
#define XT_CYL_ACCUMULATED_EVAL 2           /* eof.accumulated_eval           (eof.py:874) */

/* where a pointer lives, for kernels (xt_pointer_access) */
#define XT_PTR_DEVICE 0       /* device or managed memory                              */
#define XT_PTR_PINNED 1       /* page-locked host memory, addressed by kernels directly */
#define XT_PTR_PAGEABLE 2     /* other host memory the device addresses (pageable access) */
#define XT_PTR_INACCESSIBLE 3 /* host memory the device cannot address                 */

/* --------------------------------------------------------------- misc */
int xt_abi_version(void);
const char *xt_last_error(void);
/* XT_PTR_* class of p on the current device.  No counterpart in the reference
 * (it has no device); used to pass host arrays straight to the kernels. */
int xt_pointer_access(const void *p);
/* ncopy asynchronous copies dst[i] <- src[i] of bytes[i] bytes on `stream`
 * (one cudaMemcpyAsync each, direction from the pointers), and a stream
 * synchronisation.  No counterpart in the reference; they let a host caller
 * collect several results with one call. */
int xt_copy_async(int ncopy, void *const *dst, const void *const *src, const size_t *bytes, void *stream);
int xt_stream_sync(void *stream);

/* --------------------------------------------------------------- spherical (SL) */
/* Upload an SL basis: replaces the per-call table reads of
 * halo_methods.read_cached_table + init_table (halo_methods.py:96,178) done by
 * spheresl.compute_coefficients_solitary (spheresl.py:587-588).
 * ev: (lmax+1) x nmax, ef: (lmax+1) x nmax x numr, xi/p0/d0: numr; host arrays. */
int xt_sph_table_create(int lmax, int nmax, int numr, int cmap, double rmin, double rmax, double scale,
                        const double *xi, const double *p0, const double *d0, const double *ev,
                        const double *ef, void **handle);
int xt_sph_table_destroy(void *handle);

/* Coefficient accumulation, spheresl.compute_coefficients_solitary
 * (spheresl.py:567-656): expcoef_out ((lmax+1)^2 x nmax, row-major) =
 * sum over particles.  Particles x, y, z, m: n float64 each. */
size_t xt_sph_accumulate_workspace(void *handle);
int xt_sph_accumulate(void *handle, const double *x, const double *y, const double *z, const double *m,
                      long long n, int no_odd, int precision, double *expcoef_out, void *workspace,
                      size_t workspace_bytes, void *stream);

/* Allocation-free variant of xt_sph_accumulate; no counterpart in the
 * reference.  For callers that cannot allocate device memory for a
 * workspace: an application or framework that owns all device memory
 * through its own pool, a latency-critical loop that cannot afford the
 * synchronisation cudaMalloc/cudaFree may cause, or a C / cgo / Fortran
 * binding with no device allocator.  The deposit grid lives in a static
 * 2 MiB device array inside the library (held on every GPU that loads it
 * until exit), so the call allocates nothing; inputs and the output are
 * still caller-owned device pointers.  Limit: (lmax+1)^2 * numr <= 262144
 * doubles, larger tables return XT_ERR_ARG.  The first call on each device
 * looks up the array's address (cudaGetSymbolAddress), and so does the first
 * call after the device's context changed (cudaDeviceReset); make those
 * calls before any stream capture.  All calls share the one array, which
 * keeps the last call's contents (each call zeroes what it uses first), so
 * calls that overlap on the GPU (concurrent streams) race: serialise them. */
int xt_sph_accumulate_noalloc(void *handle, const double *x, const double *y, const double *z,
                              const double *m, long long n, int no_odd, int precision, double *expcoef_out,
                              void *stream);

/* Contract coefficients (scaled by `coef_scale`, e.g. Fields.halofac) with
 * the radial tables into an evaluation field (kept in `field`, caller-owned).
 * lmax_use/nmax_use truncate the expansion (spheresl.py:1139-1151). */
size_t xt_sph_field_bytes(void *handle, int precision);
int xt_sph_prepare(void *handle, const double *expcoef, double coef_scale, int lmax_use, int nmax_use,
                   int precision, void *field, size_t field_bytes, void *stream);

/* Evaluate at n points (spheresl.all_eval_particles / all_eval / force_eval).
 * outs: array of 8 device pointers (may be NULL to skip):
 *   ALL_EVAL_PARTICLES: den0 den1 pot0 pot1 potr pott potp rr
 *   ALL_EVAL:           den0 den1 pot0 pot1 potr pott potp -
 *   FORCE_EVAL:         potr pott potp pot1 pot0 - - -
 * L1/L2: l range (ALL_EVAL_PARTICLES); trig_l: 1 = the reference force_eval
 * azimuthal factor cos(l phi) (spheresl.py:1173), 0 = cos(m phi). */
int xt_sph_eval_points(void *handle, const void *field, int precision, int coord_mode, const double *a,
                       const double *b, const double *c, long long n, int mode, int L1, int L2, int no_odd,
                       int lmax_use, int trig_l, double *const *outs, void *stream);

/* Batched accumulation over many snapshots in one persistent launch: the
 * coefficient time series spheresl.compute_coefficients (spheresl.py:439)
 * would produce snapshot by snapshot.  xyzm: FP32 x y z m per particle
 * (float4, 16-byte aligned), snapshot s owning particles
 * [offsets_host[s], offsets_host[s+1]) (host array of nsnap+1, starting at 0).
 * FP32 per-particle arithmetic and shared-memory accumulation per work item
 * (chunk particles x one block of coefficient rows), FP64 cross-item sums and
 * FP64 contraction.  expcoef_out: nsnap x (lmax+1)^2 x nmax.  threads: CTA
 * size (128..1024).  lmax <= 8. */
size_t xt_sph_batched_workspace(void *handle, int nsnap, long long n_total, int chunk);
int xt_sph_accumulate_batched(void *handle, const float *xyzm, const long long *offsets_host, int nsnap,
                              int no_odd, int chunk, int threads, double *expcoef_out, void *workspace,
                              size_t workspace_bytes, void *stream);

/* The batched accumulation above on the tensor cores, the same sums written
 * as particles x basis-terms products: spheresl.compute_coefficients
 * (spheresl.py:439-475, accumulation loop :598-654) for every snapshot of a
 * time series.  Particles are counting-sorted by (snapshot, window of 127
 * radial table intervals); for each window, D[node, row] = sum over particles
 * of W^T[node, p] A[p, row] (W: the two interpolation weights -4 pi m plerp
 * {x1, x2} of each particle; A: its angular basis values fact P_l^m
 * {1, cos m phi, sin m phi}) runs as tcgen05 MMAs with BF16 operands and FP32
 * accumulation in tensor memory (M = 128 nodes, N = rows padded to 16,
 * K = particles); window partials are summed in FP64 and contracted with the
 * radial tables in FP64.  Same arguments as xt_sph_accumulate_batched, with
 * chunk = the most particles of one work item (>= 128), stages = operand
 * buffers per CTA (1 to 3; fewer buffers let more CTAs share an SM) and
 * ctas_per_sm = CTAs of the persistent launch per SM (0: as many as are
 * resident; xt_sph_batched_tc_residency gives that number for a depth) and
 * threads_per_particle = 1 or 2 (2: the angular rows of a particle are split
 * by the parity of m between two threads, twice the threads per CTA).
 * numr <= 8129, lmax <= 8, at most 2^31 - 1 particles.  The workspace size
 * depends on the snapshot sizes.
 * xt_sph_batched_tc_status synchronises the device and reports (and clears)
 * an error flag a launch set: XT_ERR_DEVICE, else XT_OK. */
size_t xt_sph_batched_tc_workspace(void *handle, int nsnap, const long long *offsets_host, int chunk);
int xt_sph_accumulate_batched_tc(void *handle, const float *xyzm, const long long *offsets_host, int nsnap,
                                 int no_odd, int chunk, int stages, int ctas_per_sm, int threads_per_particle,
                                 double *expcoef_out, void *workspace, size_t workspace_bytes, void *stream);
int xt_sph_batched_tc_residency(void *handle, int stages, int threads_per_particle, int *ctas_per_sm);
int xt_sph_batched_tc_status(void);

/* --------------------------------------------------------------- cylindrical (EOF) */
/* Upload EOF tables parsed by eof.parse_eof (eof.py:224-313); each table is
 * (mmax+1) x norder x (numx+1) x (numy+1) float64; force tables may be NULL
 * (stored as zeros, for accumulation-only use) and dens tables may be NULL
 * when dens == 0.  XMIN/dX/YMIN/dY from eof.set_table_params (eof.py:316). */
int xt_cyl_table_create(int mmax, int norder, int numx, int numy, int cmap, int dens, double XMIN,
                        double dX, double YMIN, double dY, double ascale, double hscale, const double *potC,
                        const double *rforceC, const double *zforceC, const double *densC, const double *potS,
                        const double *rforceS, const double *zforceS, const double *densS, void **handle);
int xt_cyl_table_destroy(void *handle);

/* Coefficient accumulation, eof.accumulate (eof.py:492-640): cos_out and
 * sin_out are (mmax+1) x norder row-major. */
size_t xt_cyl_accumulate_workspace(void *handle);
int xt_cyl_accumulate(void *handle, const double *x, const double *y, const double *z, const double *m,
                      long long n, int precision, double *cos_out, double *sin_out, void *workspace,
                      size_t workspace_bytes, void *stream);

/* Contract cos/sin coefficients with the tables into an evaluation field.
 * mmax_use/nmax_use truncate (eof.py:789-799); density != 0 also contracts
 * the density tables. */
size_t xt_cyl_field_bytes(void *handle, int density, int precision);
int xt_cyl_prepare(void *handle, const double *cos_c, const double *sin_c, int mmax_use, int nmax_use,
                   int density, int precision, void *field, size_t field_bytes, void *stream);

/* Evaluate at n points.  outs (8 device pointers, NULL to skip):
 *   ACCUMULATED_EVAL_PARTICLES: p0 p fr fp fz R d0 d   (m1 <= m <= m2)
 *   FORCE_EVAL:                 fr fp fz p p0 fr0 fz0 -  (perturb != 0: fr,fz,p
 *                               exclude m = 0, as eof.py:861-867)
 *   ACCUMULATED_EVAL:           p0 p fr fp fz d0 d - */
int xt_cyl_eval_points(void *handle, const void *field, int precision, int density, int coord_mode,
                       const double *a, const double *b, const double *c, long long n, int mode, int m1, int m2,
                       int mmax_use, int no_odd, int perturb, double *const *outs, void *stream);

/* Accumulate and evaluate at the same particles in one pipeline:
 * eof.compute_coefficients followed by eof.compute_forces on one snapshot
 * (eof.py:1158-1317).  Writes cos_out/sin_out ((mmax+1) x norder) and outs =
 * p0 p fr fp fz R (6 device arrays of n) for m1 <= m <= m2.  Per-particle
 * set-up is computed once and particles are counting-sorted by table cell
 * inside the workspace (size from xt_cyl_accumulate_eval_workspace).
 * nan_to_origin != 0 places particles with a NaN coordinate at the origin
 * for both accumulation and evaluation (eof.py:1189-1204).  mmax <= 8,
 * norder <= 24.  Unlike the other entry points, x, y, z, m and outs may also
 * be host memory the device addresses (xt_pointer_access XT_PTR_PINNED or
 * XT_PTR_PAGEABLE): the kernels then read the particles in place over the
 * host link.  Page-locked results are evaluated in two parts of the particle
 * range (the first 3/8, then the rest) into the workspace, the first part
 * copied out on a second stream while the second is evaluated (the call's
 * stream waits for the copies); pageable
 * results are evaluated in particle order so that their writes over the link
 * are coalesced.  XT_PTR_INACCESSIBLE pointers return XT_ERR_ARG. */
size_t xt_cyl_accumulate_eval_workspace(void *handle, long long n, int precision);
int xt_cyl_accumulate_eval(void *handle, const double *x, const double *y, const double *z, const double *m,
                           long long n, int precision, int m1, int m2, int nan_to_origin, double *cos_out,
                           double *sin_out, double *const *outs, void *workspace, size_t workspace_bytes,
                           void *stream);

/* The two halves of xt_cyl_accumulate_eval as separate calls, for the
 * drop-in functions that the reference runs one at a time; workspace size from
 * xt_cyl_accumulate_eval_workspace, the same limits (mmax <= 8, norder <= 24)
 * and the same host-memory rules for x, y, z, m and outs.
 * xt_cyl_accumulate_sorted: eof.accumulate / eof.compute_coefficients
 * (eof.py:492-640, 1158-1260) by binning, counting sort by table cell,
 * run-accumulated deposit and contraction into cos_out/sin_out, which may be
 * device memory or host memory the device addresses (the last kernel then
 * writes the coefficients over the host link, with no copy behind it).
 * xt_cyl_eval_sorted: eof.accumulated_eval_particles / eof.compute_forces
 * (eof.py:989-1144, 1263-1317) without density, for m1 <= m <= m2, from the
 * coefficients cos_c/sin_c ((mmax+1) x norder, device memory or host memory
 * the device addresses, which the field stage then reads in place): binning, counting
 * sort, field and evaluation in cell order; outs = p0 p fr fp fz R (6 arrays
 * of n, any may be NULL), results in particle order. */
int xt_cyl_accumulate_sorted(void *handle, const double *x, const double *y, const double *z, const double *m,
                             long long n, int precision, int nan_to_origin, double *cos_out, double *sin_out,
                             void *workspace, size_t workspace_bytes, void *stream);
int xt_cyl_eval_sorted(void *handle, const double *x, const double *y, const double *z, long long n, int precision,
                       int m1, int m2, const double *cos_c, const double *sin_c, double *const *outs,
                       void *workspace, size_t workspace_bytes, void *stream);

/* Field stage of xt_cyl_accumulate_eval and xt_cyl_eval_sorted (the
 * potential and force tables contracted with the coefficients at every node,
 * eof.py:1100-1125 summed once per node instead of per particle).
 * xt_cyl_field_engine selects its kernel for later calls: 0 (default) the
 * bulk-copy pipeline (cp.async.bulk staging of each node block's table rows in
 * shared memory, one persistent CTA per SM) where its stages fit, else row
 * loads; 1 the pipeline (XT_ERR_ARG from the calls where it does not fit);
 * 2 row loads.  Both give the field to double-float rounding (not bit-equal:
 * the pipeline sums two halves of the orders separately).
 * xt_cyl_status synchronises the device and reports (and clears) the error
 * flag of the pipeline's bounded waits: XT_ERR_DEVICE, else XT_OK. */
int xt_cyl_field_engine(int engine);
int xt_cyl_status(void);

/* Node blocks (64 consecutive nodes of the tables) that the last
 * xt_cyl_accumulate_eval / xt_cyl_accumulate_sorted / xt_cyl_eval_sorted call
 * on `workspace` (made for n particles at `precision`) contracted and
 * evaluated: those holding a corner node of a table cell with particles;
 * the deposit grid is zero elsewhere and the evaluation reads no other node.
 * Synchronises the device; *total = all node blocks of the table.
 * Diagnostics, no counterpart in the reference. */
int xt_cyl_active_blocks(void *handle, const void *workspace, long long n, int precision, int *active, int *total);

/* The double-float functions of the FP64 binning on n device values, each
 * input rounded to a float pair and each result widened to FP64 (diagnostics,
 * for accuracy tests; no counterpart in the reference): fn 0 log x
 * (2^-125 < x < 2^126), 1 asinh x (0 <= x < 2^100), 2 the z map of
 * compatibility.z_to_y at hscale = 1, z / (|z| + 1e-8) asinh |z|
 * (compatibility.py:83-91). */
int xt_df_eval(int fn, const double *in, double *out, long long n, void *stream);

/* Stage timing (diagnostics, no counterpart in the reference): with
 * xt_timing_enable(1), xt_cyl_accumulate_eval records CUDA events on its
 * stream between its stages; xt_timing_read waits for the last one and writes
 * up to `max` stage durations in ms (binrec, scan, scatter, deposit,
 * contract, field, eval), returning how many it wrote (< 0 on error). */
int xt_timing_enable(int on);
int xt_timing_read(double *ms_out, int max);

/* --------------------------------------------------------------- fields + orbits */
/* potential.Fields.return_forces_cart (potential.py:445-497) at n points:
 * outs = fxdisk fxhalo fydisk fyhalo fzdisk fzhalo diskp halop+halop0.
 * Fields prepared with xt_sph_prepare(coef_scale = halofac, halo_use_l/n) and
 * xt_cyl_prepare(disk_use_m/n).  rotpos: per-point array or NULL (then
 * rotpos_scalar is used). */
int xt_fields_forces(void *sph, const void *sph_field, void *cyl, const void *cyl_field, int precision,
                     int halo_l, int disk_m, int no_odd, int trig_l, const double *x, const double *y,
                     const double *z, const double *rotpos, double rotpos_scalar, long long n,
                     double *const *outs, void *stream);

/* Velocity-Verlet orbits (integrate.leapfrog_integrate, integrate.py:53-190)
 * for n independent orbits.  state: 16 device arrays of n float64
 * (x y z vx vy vz fx fy fz pot r2m1 r2m2 aps nstep e0 emaxdev) updated in
 * place; steps [step0, step0+nsteps) of a run of nint steps with rotation
 * angle rotc * (k*dt) at step k.  dt_per_orbit (device, may be NULL): a step
 * size per orbit replacing dt (integrate.integrate_grid gives every orbit its
 * own compute_timestep step, integrate.py:848-884).  traj (optional, may be NULL): row-major
 * (n, nint, 10) = x y z vx vy vz p fx fy fz of every step.  apse != 0 stops
 * an orbit after ap_max planar apocentres.  The force precision follows
 * `precision` (fields prepared at that precision); kick/drift are FP64. */
int xt_leapfrog(void *sph, const void *sph_field, void *cyl, const void *cyl_field, int precision,
                int halo_l, int disk_m, int no_odd, int trig_l, double *const *state, long long n,
                int step0, int nsteps, int nint, double dt, double rotc, int apse, int ap_max, double *traj,
                const double *dt_per_orbit, void *stream);

/* Reordering of an orbit ensemble between chunks of xt_leapfrog steps (no
 * reference counterpart; the reference integrates one orbit at a time): the
 * orbits of state_in (16 x n float64, row k = state array k, contiguous) are
 * counting-sorted by the disc table cell of their position (the cell of
 * eof.return_bins, eof.py:354-427) into state_out, so that the threads of a
 * warp gather from the same table cells; order_out[q] = order_in of the orbit
 * placed at q.  xt_orbit_unsort writes state_in's orbit q to column order[q]
 * of state_out.  Each orbit's arithmetic is independent of its position, so a
 * sorted run unsorted at the end equals the unsorted run bit for bit. */
size_t xt_orbit_sort_workspace(void *cyl, long long n);
int xt_orbit_sort(void *cyl, const double *state_in, double *state_out, long long n, const long long *order_in,
                  long long *order_out, void *workspace, size_t workspace_bytes, void *stream);
int xt_orbit_unsort(const double *state_in, double *state_out, long long n, const long long *order, void *stream);

/* ------------------------------------------------------------------ learned radial basis
 * No counterpart in the reference: a surrogate for the SL radial tables of
 * spheresl (get_halo_dens_pot_force, spheresl.py:106-160).  One network per
 * harmonic l (L = lmax + 1 networks) maps t = clamp((ln r - c0) c1, -1, 1)
 * through 1 -> 128 -> 128 -> 128 -> nout (SiLU) to nout = 2K residuals
 *   Y[n]   = (phi_nl(r) - s_nl HO_nl(r/a)) / sig[l][n]
 *   Y[K+n] = (r dphi_nl/dr - s_nl r dHO_nl/dr) / sig[l][K+n]
 * over the Hernquist-Ostriker functions HO_nl.  BF16 weights (FP32 masters),
 * FP32 accumulation on the tensor cores.  Parameters per network:
 * xt_mlp_param_size() floats laid out W1[128] b1[128] W2[128][128] b2[128]
 * W3[128][128] b3[128] W4[64][128] b4[64] (W[out][in]; rows >= nout zero). */
int xt_mlp_param_size(void);
int xt_mlp_create(int L, int nout, const float *init_params, void **handle);
int xt_mlp_destroy(void *handle);
/* device scratch of one forward / training step on a batch of B (B % 64 == 0) */
size_t xt_mlp_workspace(void *handle, int B);
/* which: 0 parameters, 1 last gradients, 2 Adam first moments, 3 second moments (host copy) */
int xt_mlp_get(void *handle, int which, float *host_out);
/* replace the parameters (host array), reset Adam with step counter `step` */
int xt_mlp_set_params(void *handle, const float *host_params, long long step);
/* Y[L][B][64] = network outputs at inputs t[B] (device) */
int xt_mlp_forward(void *handle, const float *t, int B, float *Y, void *workspace, size_t workspace_bytes,
                   void *stream);
/* One step: forward, MSE over the first nout columns of T (T[l] at l * ldT,
 * rows of 64), backward, and (do_update) Adam with rate lr (beta 0.9/0.999,
 * eps 1e-8).  loss_out (device, may be NULL): L doubles, MSE per network. */
int xt_mlp_train_step(void *handle, const float *t, const float *T, long long ldT, int B, float lr, int do_update,
                      double *loss_out, void *workspace, size_t workspace_bytes, void *stream);
/* Training data from an SL table (cmap 2, lmax <= 7): inputs t[n] and
 * targets T[l][n][64] (T[l] at l * ldT) at radii r[n] (device, FP64).
 * s: (lmax+1) x K prior scales, sig: (lmax+1) x 2K target scales (device). */
int xt_mlp_labels(void *sph, int K, const double *r, long long n, double a_prior, const double *s,
                  const double *sig, double c0, double c1, float *t_out, float *T_out, long long ldT, void *stream);
/* Fold one coefficient set (expcoef (lmax+1)^2 x nmax, device FP64, times
 * coef_scale) into the networks' last layers and the prior weights. */
size_t xt_learned_prep_bytes(void *mlp, int K);
int xt_learned_prepare(void *sph, void *mlp, int K, const double *expcoef, double coef_scale, const double *s,
                       const double *sig, void *prep, size_t prep_bytes, void *stream);
/* Potential and gradient at n points (xyzw: float4 x y z -, device) in the
 * spheresl.all_eval formulation (cos/sin(m phi)); out: float4 per point =
 * (pot0 + pot1, dpot/dr, dpot/dcos(theta), dpot/dphi).  Radius band b of
 * nbands (<= 64) equal bands in ln r over the table range uses the networks
 * when band_use[b] != 0 (host int array) and FP32 table interpolation of
 * field_f32 (xt_sph_prepare at XT_F32 with the same coefficients) otherwise. */
size_t xt_learned_eval_workspace(void *sph, long long n);
int xt_learned_eval(void *sph, const void *field_f32, void *mlp, const void *prep, int K, double a_prior, double c0,
                    double c1, const int *band_use, int nbands, const float *xyzw, long long n, int no_odd,
                    int engine, float *out, void *workspace, size_t workspace_bytes, void *stream);
/* engine selects the network pass: 0 = mma.sync warp tiles, 1 = tcgen05 with
 * accumulators in tensor memory.  The network pass alone (for comparisons):
 * R[n][rstride] with rstride = 2 (lmax+1)^2 rounded up to a multiple of 4;
 * row p holds, for every coefficient row, the folded network sums (potential,
 * r d/dr) of points in network bands. */
int xt_learned_radial_pass(void *sph, void *mlp, const void *prep, int K, double a_prior, double c0, double c1,
                           const int *band_use, int nbands, const float *xyzw, long long n, int engine, float *R,
                           void *stream);
/* Synchronises, then reports (and clears) a tensor-memory pass that gave up
 * waiting for its MMAs: XT_ERR_DEVICE, else XT_OK. */
int xt_learned_status(void);

/* --------------------------------------------------------------- orbit frequencies */
/* Spectra and peaks of nsig orbit signals of n samples: signal s, sample t at
 * a[t * ld + s] (+ i b[t * ld + s] when b != NULL), times win[t] when win !=
 * NULL (numpy.hanning values); device arrays.  The n-point DFT of
 * numpy.fft.fft in double-float arithmetic, one CTA per signal: a radix-2
 * FFT of size m = n for n a power of two, else Bluestein's transform with
 * m = 2^p >= 2n - 1 (m <= 4096).  Tables as complex double-float quadruples
 * (re hi, re lo, im hi, im lo; float32, 16-byte aligned, device): tw[m/2] =
 * exp(-2 pi i t/m); chirp[n] = exp(-i pi t^2/n) and chirp_f[m] = the m-point
 * FFT of the chirp's conjugate wrapped circularly (Bluestein only, else NULL).
 * mode 0: exptool/orbits/frequencies.py:94-132 organize_frequencies on the
 * spectrum: idx_out[s][0..2] = the three strongest strict relative maxima of
 * |Re X| (order neighbours each side, ends clipped) at positive frequencies
 * (freq_sign = sign of the time step), -1 when missing, val_out = their
 * |Re X|.  mode 1: frequencies.py:135-217: idx_out[s][0] = first index of the
 * largest |X| with bin 0 set to zero when zero_first.  spec_out (may be NULL):
 * [nsig][n] complex doubles. */
int xt_orbit_spectra(int mode, long long nsig, int n, const double *a, const double *b, long long ld,
                     const double *win, int order, int zero_first, int freq_sign, int m, const float *tw,
                     const float *chirp, const float *chirp_f, int *idx_out, double *val_out, double *spec_out,
                     void *stream);

/* --------------------------------------------------------------- table generation */
/* Basis functions of the cylindrical EOF construction at npt points (R, z),
 * for azimuthal order m: psi = Phi_nl Y_lm and, with derivs != 0,
 * dpsi/dR, dpsi/dz and rho_nl Y_lm, for l = m, m+2, ..., lmax and n < nmax
 * (function index ((l - m) / 2) * nmax + n; outputs [nfunc][npt] FP64, device).
 * No counterpart in the reference, which reads EOF caches but cannot make
 * them (exptool/basis/eof.py:94-95); the Y_lm normalisation is its
 * factorial_return (spheresl.py:823-863).  Radial functions from the cubic
 * spline of u_nl(t = ln r): knots [nseg+1], coef [lmax+1][nseg][nmax][4]
 * (descending powers of t - knot), Phi_nl = u Phi0 inv_sqrt_ev,
 * rho_nl = u rho0 sqrt_ev ([lmax+1][nmax] each); phi0, dphi0, rho0: the
 * background model at r = max(sqrt(R^2 + z^2), rmin).  All arrays device. */
int xt_eof_basis(int m, int lmax, int nmax, int nseg, const double *knots, const double *coef,
                 const double *inv_sqrt_ev, const double *sqrt_ev, const double *R, const double *z,
                 const double *phi0, const double *dphi0, const double *rho0, double rmin, long long npt, int derivs,
                 double *psi, double *dR, double *dz, double *rho, void *stream);

/* --------------------------------------------------------------- snapshot records */
/* Column kinds of xt_records_to_columns: source field -> column element. */
#define XT_COL_F32 0         /* float  -> float            */
#define XT_COL_F64 1         /* double -> double           */
#define XT_COL_I32 2         /* int32  -> int32            */
#define XT_COL_I64 3         /* int64  -> int64            */
#define XT_COL_F32_TO_F64 4  /* float  -> double           */

/* De-interleave n packed particle records of rec_bytes bytes (a multiple of 4,
 * at most 384) into ncol (<= 32) columns: field c at byte col_off[c] (a
 * multiple of 4) of each record, converted per col_kind[c], is written to
 * outs[c][0..n).  Replaces the NumPy structured memmap + per-field copies of
 * exptool/io/psp_io.py:196-230 and spl_io.py:235-270.  records and outs may
 * be device memory or host memory the device addresses (xt_pointer_access);
 * col_off, col_kind and the outs array itself are host arrays. */
int xt_records_to_columns(const void *records, long long n, int rec_bytes, int ncol, const int *col_off,
                          const int *col_kind, void *const *outs, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* EXPTOOL_GB300_H */
