/*
 * chimeracl_gb300 -- C ABI of the GB300 (sm_103a) kernels behind the
 * quasi-cylindrical PSATD particle-in-cell step.
 *
 * Every entry point replaces one method (or one fused group of methods) of
 * chimeraCL's methods layer (chimeraCL/methods/*_methods_cl.py) and the
 * OpenCL kernels it launches; the reference file:line is given beside each.
 *
 * Conventions
 *  - All pointers are device pointers unless stated; sizes are element counts.
 *  - `dtype` selects the arithmetic: CCL_F64 (the plain FP64 drop-in: double
 *    particles, double/complex128 fields) or CCL_F32 (float particles,
 *    float/complex64 fields).  Complex arrays are interleaved (re, im).
 *    "Real coefficient" arrays (filters, PSATD coefficients, 1/dV, damping
 *    profile) are in the same real type as `dtype`; knot, grid and theta
 *    arrays of the plasma injector are always double.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    asynchronous on that stream; none synchronises the host.
 *  - Return value: CCL_OK (0) or an error code; ccl_last_error() gives a
 *    message.  Arguments are validated before any launch.
 */
#ifndef CHIMERACL_GB300_H
#define CHIMERACL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CCL_OK 0
#define CCL_ERR_ARG 1         /* invalid argument (null pointer, bad size) */
#define CCL_ERR_CUDA 2        /* a CUDA launch or runtime call failed */
#define CCL_ERR_UNSUPPORTED 3 /* a size or mode this library does not handle */
#define CCL_ERR_WORKSPACE 4   /* workspace smaller than required */

#define CCL_F64 0
#define CCL_F32 1

/* Library version (major*10000 + minor*100 + patch). */
int ccl_version(void);
/* Message of the last error returned on the calling thread. */
const char *ccl_last_error(void);
/* Number of kernels this library has launched since it was loaded. */
unsigned long long ccl_launch_count(void);

/* ------------------------------------------------------------------ */
/* Particles  (chimeraCL/methods/particles_methods_cl.py)              */
/* ------------------------------------------------------------------ */

/* x += px*dt*g_inv (same for y, z) for np particles.
 * Replaces push_coords -> push_xyz (particles_methods_cl.py:206-223,
 * kernels/particles_generic.cl:129-153); dt is the species' dt_2 or dt. */
int ccl_push_x(int dtype, long np, void *x, void *y, void *z, const void *px,
               const void *py, const void *pz, const void *g_inv, double dt,
               void *stream);

/* The same push with each coordinate held as the unevaluated sum hi + lo
 * (x + x_lo, ...): the displacement of push_xyz is added by a two-sum into
 * the low part and the pair renormalised, so x stays the nearest value to
 * the compensated coordinate.  No counterpart in the reference (its
 * coordinates are FP64); it keeps FP32 coordinates from losing the
 * displacements below half a unit in the last place (a slow particle stops,
 * and its charge and current then disagree).  x_lo, y_lo, z_lo start at 0
 * for new particles. */
int ccl_push_x_compensated(int dtype, long np, void *x, void *y, void *z, void *x_lo,
                           void *y_lo, void *z_lo, const void *px, const void *py,
                           const void *pz, const void *g_inv, double dt, void *stream);

/* Bytes of device workspace ccl_index_sort needs for np particles on a grid
 * of ncells = (Nx-1)*(Nr-1) cells. */
int ccl_index_sort_workspace(long np, long ncells, size_t *bytes);

/* Cell index and cell sort of np particles.
 * Replaces index_sort (particles_methods_cl.py:225-261): the kernels
 * index_and_sum_in_cell (particles_generic.cl:88-126) and sort
 * (particles_generic.cl:186-201) and the cumsum between them.
 * Outputs, all exact integers:
 *   indx_in_cell[np]        key = ix + ir*(Nx-1) for 0<ix<Nx-2, 0<=ir<Nr-2,
 *                           else the overflow key (Nx-1)*(Nr-1);
 *   sum_in_cell[C+1]        particles per key, C = (Nx-1)*(Nr-1);
 *   cell_offset[C+2]        exclusive prefix sum, cell_offset[0] = 0;
 *   sort_indx[np]           particle numbers in key order -- the sort is
 *                           stable, so within a cell in ascending order;
 *   np_stay[1] (device)     cell_offset[C], the in-window count.
 * The host reads nothing; np_stay stays on the device.  The offsets come
 * from a single-pass scan whose tiles wait (bounded) on their predecessors'
 * sums; ccl_sort_status reports a wait that gave up. */
int ccl_index_sort(int dtype, long np, const void *x, const void *y,
                   const void *z, int Nx, double xmin, double dx_inv, int Nr,
                   double rmin, double dr_inv, uint32_t *indx_in_cell,
                   uint32_t *sum_in_cell, uint32_t *cell_offset,
                   uint32_t *sort_indx, uint32_t *np_stay, void *workspace,
                   size_t workspace_bytes, void *stream);

/* The same sort in two calls around the coordinate push, so that the keys
 * are formed from the coordinates the push has just computed instead of
 * being read back: ccl_push_x_keys runs push_xyz (ccl_push_x, or with
 * x_lo, y_lo, z_lo non-null ccl_push_x_compensated) and the first pass of
 * ccl_index_sort (indx_in_cell, sum_in_cell, per-tile counts kept in the
 * workspace, and the workspace's cursors and scan flags cleared);
 * ccl_index_sort_keyed, on the same workspace before any other
 * use of it, completes the sort (cell_offset, sort_indx, np_stay); run
 * again with no key pass in between, its scan finds the workspace not
 * cleared and sets ccl_sort_status (nothing is written out of bounds).  The
 * outputs are those of ccl_push_x followed by ccl_index_sort.  Replaces the
 * pair push_coords + sort_parts of the reference's loop (pic_loop.py:74-98,
 * particles_methods_cl.py:206-261) with no counterpart of its own. */
int ccl_push_x_keys(int dtype, long np, void *x, void *y, void *z, void *x_lo, void *y_lo,
                    void *z_lo, const void *px, const void *py, const void *pz,
                    const void *g_inv, double dt, int Nx, double xmin, double dx_inv, int Nr,
                    double rmin, double dr_inv, uint32_t *indx_in_cell, uint32_t *sum_in_cell,
                    void *workspace, size_t workspace_bytes, void *stream);
int ccl_index_sort_keyed(long np, int Nx, int Nr, const uint32_t *indx_in_cell,
                         uint32_t *sum_in_cell, uint32_t *cell_offset, uint32_t *sort_indx,
                         uint32_t *np_stay, void *workspace, size_t workspace_bytes,
                         void *stream);

/* ccl_index_sort without a caller-owned workspace.  No counterpart in the
 * reference: it is for callers that cannot allocate device memory for the
 * sort (a host binding that owns no device allocator, or a process whose
 * device memory is reserved up front by another framework).  The workspace is
 * a file-scope 9 MiB device array -- enough for up to 2,000,000 cells with up
 * to 2^26 particles; larger inputs return CCL_ERR_WORKSPACE without
 * launching anything.  Each call outside a stream capture looks up the
 * array's device address on the calling device (cudaGetSymbolAddress); a
 * call inside a capture reuses the last one, so the first call on a device
 * must come before any stream capture (inside one it returns
 * CCL_ERR_UNSUPPORTED).  Nothing is allocated.  Calls that overlap in time on one device
 * (other streams, other host threads) share the array and race; outputs
 * and their meaning are those of ccl_index_sort. */
int ccl_index_sort_noalloc(int dtype, long np, const void *x, const void *y,
                           const void *z, int Nx, double xmin, double dx_inv,
                           int Nr, double rmin, double dr_inv,
                           uint32_t *indx_in_cell, uint32_t *sum_in_cell,
                           uint32_t *cell_offset, uint32_t *sort_indx,
                           uint32_t *np_stay, void *stream);

/* dst[c][i] = src[c][sort_indx[i]] for i < n, c < ncomp (ncomp <= 16).
 * `src`, `dst` are host arrays of ncomp device pointers.
 * Replaces align_and_damp -> data_align_dbl (particles_methods_cl.py:263-286,
 * particles_generic.cl:156-169). */
int ccl_align(int dtype, long n, int ncomp, void *const *src, void *const *dst,
              const uint32_t *sort_indx, void *stream);

/* a[i] = i for i < n (the sort_indx reset of align_and_damp,
 * particles_methods_cl.py:283-285). */
int ccl_iota_u32(uint32_t *a, long n, void *stream);

/* Fill ncells = (Nx_loc-1)*(Nr_loc-1) cells with Nppc = npx*npr*npth
 * particles each; w = r.  Replaces make_new_domain -> fill_grid
 * (particles_methods_cl.py:66-98, particles_generic.cl:33-84). theta, xgrid,
 * rgrid are double device arrays. */
int ccl_fill_grid(int dtype, long ncells, void *x, void *y, void *z, void *w,
                  const double *theta, const double *xgrid,
                  const double *rgrid, uint32_t Nx_loc, uint32_t npx,
                  uint32_t npr, uint32_t npth, void *stream);

/* w[i] *= f(x[i]), f piecewise linear on nloc knots xx/ff (double),
 * dxm1 = 1/(xx[k+1]-xx[k]).  Replaces dens_profile -> profile_by_interpolant
 * (particles_methods_cl.py:179-204, particles_generic.cl:6-30). */
int ccl_dens_profile(int dtype, long np, const void *x, void *w,
                     const double *xx, const double *ff, const double *dxm1,
                     uint32_t nloc, void *stream);

/* g_inv = 1/sqrt(1 + px^2 + py^2 + pz^2)
 * (particles_methods_cl.py:141-144, 174-177). */
int ccl_gamma_inv(int dtype, long np, const void *px, const void *py,
                  const void *pz, void *g_inv, void *stream);

/* ------------------------------------------------------------------ */
/* Grid  (chimeraCL/methods/grid_methods_cl.py)                        */
/* ------------------------------------------------------------------ */

/* rho_m += sum over sorted particles of q*w*S(x)S(r) e^{i m phi},
 * m = 0..M; rho is a host array of M+1 device pointers (m=0 real (Nr,Nx),
 * m>=1 complex (Nr,Nx)).  Replaces depose_scalar (grid_methods_cl.py:44-69,
 * grid_deposit_m0.cl:20-129, grid_deposit_m1.cl:20-152). */
int ccl_deposit_scalar(int dtype, int M, const uint32_t *sort_indx,
                       const uint32_t *cell_offset, const void *x,
                       const void *y, const void *z, const void *w, int charge,
                       int Nx, double xmin, double dx_inv, int Nr, double rmin,
                       double dr_inv, void *const *rho, void *stream);

/* J_k,m += q*w*g_inv*u_k*S(x)S(r) e^{i m phi}; J is a host array of 3*(M+1)
 * device pointers ordered m-major then x,y,z.  Replaces depose_vector
 * (grid_methods_cl.py:71-95, grid_deposit_m0.cl:148-277,
 * grid_deposit_m1.cl:171-327). */
int ccl_deposit_vector(int dtype, int M, const uint32_t *sort_indx,
                       const uint32_t *cell_offset, const void *x,
                       const void *y, const void *z, const void *ux,
                       const void *uy, const void *uz, const void *g_inv,
                       const void *w, int charge, int Nx, double xmin,
                       double dx_inv, int Nr, double rmin, double dr_inv,
                       void *const *J, void *stream);

/* The two deposits for FP32 particles whose coordinates are held as
 * hi + lo (x + x_lo, ...; see ccl_push_x_compensated): the cell and the
 * angle come from x, y, z, the shape-function fractions from the full
 * coordinates (the cell edge and the radius formed as float pairs), so they
 * resolve a 2^-24 fraction of a cell however far the coordinate is from 0.
 * No counterpart in the reference (its coordinates are FP64).  dtype must
 * be CCL_F32. */
int ccl_deposit_scalar_lo(int dtype, int M, const uint32_t *sort_indx,
                          const uint32_t *cell_offset, const void *x, const void *y,
                          const void *z, const void *w, int charge, int Nx, double xmin,
                          double dx_inv, int Nr, double rmin, double dr_inv, void *const *rho,
                          const void *x_lo, const void *y_lo, const void *z_lo, void *stream);
int ccl_deposit_vector_lo(int dtype, int M, const uint32_t *sort_indx,
                          const uint32_t *cell_offset, const void *x, const void *y,
                          const void *z, const void *ux, const void *uy, const void *uz,
                          const void *g_inv, const void *w, int charge, int Nx, double xmin,
                          double dx_inv, int Nr, double rmin, double dr_inv, void *const *J,
                          const void *x_lo, const void *y_lo, const void *z_lo, void *stream);

/* Axis treatment (row 1 -= row 0) then multiplication by dV_inv[ir] for
 * nfld fields of M+1 modes (flds: nfld*(M+1) pointers, field-major).
 * Replaces postproc_depose_scalar / postproc_depose_vector
 * (grid_methods_cl.py:98-151, grid_generic.cl:4-59). */
int ccl_deposit_postproc(int dtype, int M, int nfld, void *const *flds,
                         int Nx, int Nr, const void *dV_inv, void *stream);

/* Ghost row 0 = +row 1 (m=0) or -row 1 (m>=1) for nfld fields.
 * Replaces preproc_project_vec (grid_methods_cl.py:153-166,
 * grid_generic.cl:63-86). */
int ccl_warp_axis(int dtype, int M, int nfld, void *const *flds, int Nx,
                  void *stream);

/* Field gather from E, B (flds: 6*(M+1) pointers, m-major then
 * Ex,Ey,Ez,Bx,By,Bz) and Boris push of u, g_inv, for the np particles of
 * sort_indx; particles with number >= *np_stay are skipped as in the
 * reference.  factor_push = 2 pi dt q/m.  Replaces _gather_and_push
 * (grid_methods_cl.py:168-192, grid_deposit_m0.cl:280-427,
 * grid_deposit_m1.cl:330-511). */
int ccl_gather_push(int dtype, int M, long np, const void *x, const void *y,
                    const void *z, void *px, void *py, void *pz, void *g_inv,
                    const uint32_t *sort_indx, const uint32_t *np_stay,
                    double factor_push, int Nx, double xmin, double dx_inv,
                    int Nr, double rmin, double dr_inv,
                    const void *const *flds, void *stream);

/* ccl_gather_push with the cell offsets of the sort (cell_offset from
 * ccl_index_sort, which the reference's gather does not take): the FP32 form
 * then runs tile by tile (32 x 8 cells per CTA, the tile's E and B staged in
 * shared memory, the tile's particles taken in sort order); the FP64 form is
 * ccl_gather_push.  Same outputs and skip rules. */
int ccl_gather_push_cells(int dtype, int M, long np, const void *x, const void *y,
                          const void *z, void *px, void *py, void *pz, void *g_inv,
                          const uint32_t *sort_indx, const uint32_t *cell_offset,
                          const uint32_t *np_stay, double factor_push, int Nx,
                          double xmin, double dx_inv, int Nr, double rmin,
                          double dr_inv, const void *const *flds, void *stream);

/* The same gather for FP32 coordinates held as hi + lo: interpolation
 * fractions from the full coordinates, as in ccl_deposit_scalar_lo.  dtype
 * must be CCL_F32. */
int ccl_gather_push_cells_lo(int dtype, int M, long np, const void *x, const void *y,
                             const void *z, void *px, void *py, void *pz, void *g_inv,
                             const uint32_t *sort_indx, const uint32_t *cell_offset,
                             const uint32_t *np_stay, double factor_push, int Nx, double xmin,
                             double dx_inv, int Nr, double rmin, double dr_inv,
                             const void *const *flds, const void *x_lo, const void *y_lo,
                             const void *z_lo, void *stream);

/* ------------------------------------------------------------------ */
/* Spectral transforms  (chimeraCL/methods/transformer_methods_cl.py)  */
/* ------------------------------------------------------------------ */

/* phs[ix] = exp(sign * i kx[ix] x0) (kx double).  Replaces get_phase_plus /
 * get_phase_minus (transformer_generic.cl:28-55). */
int ccl_phase(int dtype, int nx, void *phs, const double *kx, double x0,
              int sign, void *stream);

/* Batched longitudinal FFT, forward stage of a transform: row r of `in`
 * (complex, or real when in_real, leading dimension in_ld elements) is
 * Fourier transformed along x (unnormalised, e^{-i}), multiplied by phs[ix]
 * and, if filter != NULL, by filter[r*nx+ix]; written to `out` (complex,
 * (nrows, nx)).  Replaces the FFT + multiply_by_phase half of
 * _transform_forward / _half_transform_forward
 * (transformer_methods_cl.py:290-333, 427-455) and fields_smooth (:79-85).
 * nx must factor into 2, 3, 5, 7 (nx <= 8192 f32, 4096 f64). */
int ccl_fft_forward_rows(int dtype, int nrows, int nx, const void *in,
                         long in_ld, int in_real, void *out, const void *phs,
                         const void *filter, void *stream);

/* Backward stage: row r of the complex spectral `in` (nrows, nx) is
 * multiplied by phs[ix], inverse transformed (normalised 1/nx, e^{+i}) and
 * written to `out` (complex, or its real part when out_real; leading
 * dimension out_ld).  Replaces the multiply_by_phase + FFT + cast half of
 * _transform_backward / _half_transform_backward
 * (transformer_methods_cl.py:334-425). */
int ccl_fft_backward_rows(int dtype, int nrows, int nx, const void *in,
                          void *out, long out_ld, int out_real,
                          const void *phs, void *stream);

/* Absorbing-edge round trip of one spectral field in place: half backward
 * transform (phase phs_plus, inverse FFT; real part for a real mode) into the
 * real-space field rows 1..nrows of `rs` ((nrows+1, nx), complex or real per
 * rs_real), edge profile (x[ix] *= f[ix] for ix < nf, x[ix] *= f[nx-ix] for
 * ix > nx-nf, also applied to rs row 0), then half forward transform (FFT,
 * phase phs_minus) back into `spec`.  Replaces damp_fields for one component
 * (solver.py:32-35, transformer_methods_cl.py:385-455,
 * solver_methods_cl.py:64-83, solver_ms_pic.cl:5-55). */
int ccl_damp_rows(int dtype, int nrows, int nx, void *spec, void *rs,
                  int rs_real, const void *phs_plus, const void *phs_minus,
                  const void *profile, int nf, void *stream);

/* Batched forms of the three row transforms above: `batch` (<= 32) entries
 * of nrows rows each, one launch.  in/out/filter/spec/rs are host arrays of
 * `batch` device pointers (filter may be NULL, or hold NULL entries);
 * in_ld/out_ld and in_real/out_real/rs_real are host arrays of `batch`
 * values.  The phase and profile arrays are shared by all entries.  Used to
 * transform every field component and mode of a step stage at once
 * (transformer.py:17-26 loops over them one transform at a time). */
int ccl_fft_forward_batch(int dtype, int batch, int nrows, int nx,
                          const void *const *in, const long *in_ld,
                          const int *in_real, void *const *out,
                          const void *phs, const void *const *filter,
                          void *stream);
int ccl_fft_backward_batch(int dtype, int batch, int nrows, int nx,
                           const void *const *in, void *const *out,
                           const long *out_ld, const int *out_real,
                           const void *phs, void *stream);
int ccl_damp_batch(int dtype, int batch, int nrows, int nx, void *const *spec,
                   void *const *rs, const int *rs_real, const void *phs_plus,
                   const void *phs_minus, const void *profile, int nf,
                   void *stream);

/* Discrete Hankel transform / spectral radial derivative as a batched GEMM:
 * Y[b] = beta*Y[b] + alpha * (A[b] X[b]) for b < batch, A[b] real (m x k,
 * row-major, lda = k), X[b] (k x ncols) with leading dimension ldx, Y[b]
 * (m x ncols), leading dimension ldy.  ncols counts real columns; when
 * cplx != 0 the columns are interleaved (re, im) pairs and alpha is the
 * complex (alpha_re, alpha_im), else alpha_re alone.  beta is 0 or 1.
 * A, X, Y are host arrays of `batch` device pointers (batch <= 32).
 * Replaces _ddot / _cdot (Reikna MatrixMul, transformer_methods_cl.py:458-480)
 * in the forward/backward transforms, field_grad and field_rot. */
int ccl_dht_gemm(int dtype, int batch, int m, int k, int ncols, int cplx,
                 const void *const *A, const void *const *X, long ldx,
                 void *const *Y, long ldy, double alpha_re, double alpha_im,
                 double beta, void *stream);

/* ccl_dht_gemm with a column count and leading dimensions per entry
 * (ncols, ldx, ldy: host arrays of `batch` values), so the real m=0 and the
 * complex m>=1 Hankel transforms of a field group share one launch. */
int ccl_dht_gemm_batch(int dtype, int batch, int m, int k, const int *ncols,
                       int cplx, const void *const *A, const void *const *X,
                       const long *ldx, void *const *Y, const long *ldy,
                       double alpha_re, double alpha_im, double beta,
                       void *stream);

/* BF16x3 form of the Hankel GEMM on the tensor cores (tcgen05, FP32
 * accumulation), for FP32 operands: A = A_hi + A_lo and X = X_hi + X_lo in
 * bf16, A X ~ A_hi X_hi + A_hi X_lo + A_lo X_hi (relative error ~1e-5).
 * The constant matrix is split once: ccl_dht_bf16x3_prepare writes the
 * split, tiled form of A (m x k, row-major, m, k <= 512, dtype CCL_F64 or
 * CCL_F32) into `out` (ccl_dht_bf16x3_prepare_bytes bytes, 16-byte aligned).
 * ccl_dht_bf16x3_gemm_batch then takes prepared matrices and the arguments
 * of ccl_dht_gemm_batch (X rows 16-byte aligned: ldx % 4 == 0).
 * ccl_dht_bf16x3_status returns (and with reset != 0 clears) the kernels'
 * device error flag: 0 = ok, else a bounded wait gave up (the kernel then
 * skipped its work and released its tensor memory).  It synchronises. */
int ccl_dht_bf16x3_prepare_bytes(int m, int k, size_t *bytes);
int ccl_dht_bf16x3_prepare(int dtype, const void *A, int m, int k, void *out,
                           size_t bytes, void *stream);
int ccl_dht_bf16x3_gemm_batch(int batch, int m, int k, const int *ncols,
                              int cplx, const void *const *A_prepared,
                              const void *const *X, const long *ldx,
                              void *const *Y, const long *ldy, double alpha_re,
                              double alpha_im, double beta, void *stream);
int ccl_dht_bf16x3_status(int reset);

/* Failure-detection check, no counterpart in the reference (which has no
 * device waits): the tensor-core GEMM's bounded mbarrier wait on a barrier
 * that nothing arrives on (arrive == 0) or that one arrival completes
 * (arrive != 0), polled at most `spins` times (1 <= spins <= 20,000,000,
 * about a second).  Writes 1 to the device int *gave_up when the wait ran
 * out and 0 when it completed; the context stays usable either way. */
int ccl_wait_probe(long spins, int arrive, int *gave_up, void *stream);

/* The cell sort's device error flag, no counterpart in the reference: the
 * single-pass scan of the cell offsets (ccl_index_sort, ccl_index_sort_keyed)
 * waits, bounded, for the sums of the tiles before its own; 0 = ok, else a
 * wait gave up (that scan's offsets are then wrong).  reset != 0 clears it.
 * It synchronises.  ccl_scan_wait_probe runs that bounded wait on its own:
 * one tile of the scan looks back at a predecessor whose sum is published
 * (publish != 0) or never written, polling at most `spins` times
 * (1 <= spins <= 1,048,576); it writes 1 to the device int *gave_up when the
 * wait ran out, else 0, and the tile's offset to scratch[6] (5 when the
 * predecessor published, 0 when not); scratch: 8 device words, 8-byte
 * aligned.  The context stays usable either way. */
int ccl_sort_status(int reset);
int ccl_scan_wait_probe(long spins, int publish, int *gave_up, uint32_t *scratch,
                        void *stream);

/* PSATD update of E and G in one azimuthal mode over ncells spectral cells.
 * flds: 15 complex device pointers E_x,E_y,E_z, G_x,G_y,G_z, J_x,J_y,J_z,
 * dN0_x..z, dN1_x..z; c1 = cos(w dt), c2 = sin(w dt) w, c3 = 1/w^2 (real).
 * Replaces advance_fields -> advance_e_g_m (solver_methods_cl.py:43-62,
 * solver_ms_pic.cl:57-143). */
int ccl_psatd_advance(int dtype, long ncells, double dt_inv, const void *c1,
                      const void *c2, const void *c3, void *const *flds,
                      void *stream);

/* The same update with cancellation-free coefficients, for FP32 fields
 * (the FP32 form's advance_fields).  coef[8*i .. 8*i+7] per spectral cell,
 * formed in double with x = w dt:
 *   cos x, w sin x, s = sin x / w, 2 pi s, 2 pi (1 - cos x),
 *   2 pi (cos x - sin x / x) / w^2, 2 pi (sin x / x - 1) / w^2,
 *   2 pi (1 - cos x) / (w^2 dt)
 * (the last three by their Taylor series for small x; the array 16-byte
 * aligned); then
 *   E1 = c1 E0 + s G0 - 2 pi s J + a N0 + b N1,
 *   G1 = -c2 E0 + c1 G0 + q J + d (N0 - N1) - 2 pi s N0.
 * Algebraically ccl_psatd_advance; the reference's grouping forms the
 * small charge and current terms of long-wavelength modes (w dt ~ 1e-3)
 * as differences of O(1) terms, which keep only 1-2 digits in FP32. */
int ccl_psatd_advance_split(int dtype, long ncells, const void *coef, void *const *flds,
                            void *stream);

/* out[ir, ix] = (-Re, +Im) of in[ir, (nx-ix) mod nx]: the m=-1 mirror.
 * Replaces _get_mm1_vec/_scl -> get_m1 (transformer_methods_cl.py:265-288,
 * transformer_generic.cl:3-24). */
int ccl_get_m1(int dtype, int nrows, int nx, void *out, const void *in,
               void *stream);

/* Combine step of the spectral gradient (field_grad,
 * transformer_methods_cl.py:87-133) for all modes at once, given the radial
 * derivative products from one batched GEMM: Pm[m] = dDHT_minus_m rho_{m-1}
 * (for m = 0: dDHT_minus_0 rho_{+1}, taken through the m=-1 mirror here),
 * Pp[m] = dDHT_plus_m rho_{m+1}; entries NULL where absent (host arrays of
 * M+1 device pointers, or NULL).  Writes dN[3m+c] = (i kx rho_m,
 * -T- + T+, -i(T- + T+)), c = x, y, z (complex (nrows, nx)). */
int ccl_grad_combine(int dtype, int M, int nrows, int nx, const void *kx,
                     const void *const *rho, const void *const *Pm,
                     const void *const *Pp, void *const *dN, void *stream);

/* Combine step of the spectral curl (field_rot,
 * transformer_methods_cl.py:185-263) for all modes, given the products
 * Qm[3m+c] = dDHT_minus_m G_{c,m-1} (m = 0: of G_{c,+1}, mirrored here) and
 * Qp[3m+c] = dDHT_plus_m G_{c,m+1}; poiss (M+1 real arrays, or NULL)
 * multiplies the result by 1/w^2 (field_poiss_vec, :66-71).  Writes B[3m+c]. */
int ccl_rot_combine(int dtype, int M, int nrows, int nx, const void *kx,
                    const void *const *G, const void *const *Qm,
                    const void *const *Qp, const void *const *poiss,
                    void *const *B, void *stream);

/* ------------------------------------------------------------------ */
/* Elementwise  (chimeraCL/methods/generic_methods_cl.py, generic.cl)  */
/* ------------------------------------------------------------------ */

/* a[i] = val for n elements (complex when cplx: (re, im)).
 * Replaces set_to (generic_methods_cl.py:96-105). */
int ccl_set(int dtype, int cplx, long n, void *a, double re, double im,
            void *stream);
/* ccl_set over `narr` arrays (narr <= 32) in one launch: array i has n[i]
 * elements at a[i], complex when cplx[i].  For the zeroing of the deposit
 * targets (grid.py:23-54), one launch instead of one per array and mode. */
int ccl_set_batch(int dtype, int narr, const int *cplx, const long *n,
                  void *const *a, double re, double im, void *stream);
/* base += add (complex n).  append_c2c, generic.cl:18-29. */
int ccl_append_c2c(int dtype, long n, void *base, const void *add,
                   void *stream);
/* z += a x (complex n).  zpaxz_c2c, generic.cl:32-44. */
int ccl_zpaxz(int dtype, long n, void *z, double are, double aim,
              const void *x, void *stream);
/* z = a x + b y (complex n).  axpbyz_c2c, generic.cl:61-77. */
int ccl_axpbyz(int dtype, long n, double are, double aim, const void *x,
               double bre, double bim, const void *y, void *z, void *stream);
/* z *= x, x real, z complex (n).  mult_elementwise_d2c, generic.cl:47-58. */
int ccl_mult_elementwise(int dtype, long n, const void *x, void *z,
                         void *stream);
/* z[ir,ix] = b[ix] * (a x[ir,ix]) over (nrows, nx), b real.
 * ab_dot_x, generic.cl:82-99. */
int ccl_ab_dot_x(int dtype, int nrows, int nx, double are, double aim,
                 const void *b, const void *x, void *z, void *stream);
/* out = Re(in) (n).  cast_array_d2c, generic.cl:102-112. */
int ccl_cast_c2d(int dtype, long n, const void *in, void *out, void *stream);
/* Edge profile on a (nrows, nx) field, in place.  profile_edges_c/_d,
 * solver_ms_pic.cl:5-55. */
int ccl_profile_edges(int dtype, int cplx, int nrows, int nx, void *a,
                      const void *f, int nf, void *stream);
/* a *= phs[ix] over complex (nrows, nx).  multiply_by_phase,
 * transformer_generic.cl:58-80. */
int ccl_multiply_by_phase(int dtype, int nrows, int nx, void *a,
                          const void *phs, void *stream);

/* ------------------------------------------------------------------ */
/* Adjoint of the step (reverse mode: gradients of a loss of the final */
/* fields with respect to the laser and the density profile).  The     */
/* reference has no adjoint: each entry point is the transpose of the  */
/* forward operation cited, for the same particles and cells (the      */
/* forward's cell sort is reused).  Adjoints of complex arrays are     */
/* stored like the arrays, (dL/dRe, dL/dIm).                           */
/* ------------------------------------------------------------------ */

/* Transpose of the charge (vec = 0) or current (vec = 1) deposit
 * (grid_methods_cl.py:44-95, grid_deposit_m1.cl:20-327): a gather of the
 * node adjoints `lam` (the deposit targets' adjoints before the
 * post-processing; vec: 3(M+1) pointers m-major then x, y, z, else M+1)
 * with the shape functions and their derivatives.  Adds to lw and, when
 * lx, ly, lz are given (all or none), to the position adjoints; vec also
 * adds to lux, luy, luz, lg (adjoints of momenta and g_inv).  sort_indx,
 * cell_offset: the forward's sort at the same positions. */
int ccl_deposit_adjoint(int dtype, int vec, int M, const uint32_t *sort_indx,
                        const uint32_t *cell_offset, const void *x, const void *y,
                        const void *z, const void *ux, const void *uy, const void *uz,
                        const void *g_inv, const void *w, int charge, int Nx, double xmin,
                        double dx_inv, int Nr, double rmin, double dr_inv, void *const *lam,
                        void *lx, void *ly, void *lz, void *lw, void *lux, void *luy,
                        void *luz, void *lg, void *stream);

/* Transpose of the gather + Boris push (grid_methods_cl.py:168-192,
 * grid_deposit_m1.cl:330-511) for the particles the forward pushed (those
 * of the valid cells of cell_offset whose number is below *np_stay).  flds:
 * the real-space E, B the forward gathered (6(M+1) pointers, m-major then
 * Ex, Ey, Ez, Bx, By, Bz, after the ghost rows); lflds: their adjoints,
 * added to.  ux_old..: momenta before the push.  On entry lux, luy, luz,
 * lg hold the adjoints of the pushed momenta and g_inv; for each pushed
 * particle they become the adjoints of the momenta before the push (lg 0),
 * and lx, ly, lz are added to. */
int ccl_gather_push_adjoint(int dtype, int M, const void *x, const void *y, const void *z,
                            const void *ux_old, const void *uy_old, const void *uz_old,
                            const uint32_t *sort_indx, const uint32_t *cell_offset,
                            const uint32_t *np_stay, double factor_push, int Nx, double xmin,
                            double dx_inv, int Nr, double rmin, double dr_inv,
                            const void *const *flds, void *const *lflds, void *lx, void *ly,
                            void *lz, void *lux, void *luy, void *luz, void *lg,
                            void *stream);

/* Transpose of push_xyz (particles_methods_cl.py:206-223,
 * particles_generic.cl:129-153): lu += dt g_inv lx, lg += dt (lx . u). */
int ccl_push_x_adjoint(int dtype, long np, const void *ux, const void *uy, const void *uz,
                       const void *g_inv, const void *lx, const void *ly, const void *lz,
                       void *lux, void *luy, void *luz, void *lg, double dt, void *stream);

/* Transpose of the PSATD update (solver_methods_cl.py:43-62,
 * solver_ms_pic.cl:57-143) in one mode, with the eight coefficients per
 * cell of ccl_psatd_advance_split (both precisions' updates are this
 * linear map).  flds: 15 pointers -- lE xyz, lG xyz (in: adjoints of the
 * updated fields; out: of the fields before the update), lJ xyz (written;
 * times `filter` per cell when it is not NULL: the transpose of the
 * smoothing filter of fields_smooth, transformer_methods_cl.py:79-85),
 * lN0 xyz (written), lN1 xyz (added to). */
int ccl_psatd_adjoint(int dtype, long ncells, const void *coef, const void *filter,
                      void *const *flds, void *stream);

/* Transpose of the gradient's combine step (transformer_methods_cl.py:
 * 87-133, ccl_grad_combine), first half: from the gradient adjoints ldN
 * (3(M+1), m-major, x y z) writes lrho[m] = -i kx ldN_x (the direct term)
 * and the operands of the transposed radial products: Pm[m] (for
 * dDHT_minus_m^T; for m = 0 through the m=-1 mirror) and Pp[m] (for
 * dDHT_plus_m^T), NULL where the forward has no such term.  The products
 * are then added by ccl_modes_adjoint_accumulate (ncomp 1). */
int ccl_grad_combine_adjoint(int dtype, int M, int nrows, int nx, const void *kx,
                             const void *const *ldN, void *const *lrho, void *const *Pm,
                             void *const *Pp, void *stream);

/* Transpose of the curl's combine step with the Poisson factor
 * (transformer_methods_cl.py:185-263, 66-71, ccl_rot_combine), first
 * half: adds the direct i kx terms of the B adjoints lB to lG and writes
 * the operands Qm, Qp (3(M+1) each, NULL for absent modes) of the
 * transposed radial products, added by ccl_modes_adjoint_accumulate
 * (ncomp 3). */
int ccl_rot_combine_adjoint(int dtype, int M, int nrows, int nx, const void *kx,
                            const void *const *poiss, const void *const *lB, void *const *lG,
                            void *const *Qm, void *const *Qp, void *stream);

/* Second half of both: lo[j] += Rm[j+1] + Rp[j-1] (+ Rm[0] for j = 1)
 * per component, where Rm[m] = dDHT_minus_m^T Pm[m] and Rp[m] =
 * dDHT_plus_m^T Pp[m] (ncomp arrays per mode; NULL where absent); then
 * lo[j] *= filt[j] where filt (M+1 real arrays) is not NULL. */
int ccl_modes_adjoint_accumulate(int dtype, int M, int ncomp, int nrows, int nx,
                                 void *const *lo, const void *const *Rm,
                                 const void *const *Rp, const void *const *filt,
                                 void *stream);

/* dst[a][i] += src[a][i] for i < n[a] reals, a < narr <= 32, one launch.
 * No counterpart in the reference (the adjoint's accumulations of
 * transformed adjoints; append_c2c, generic.cl:18-29, per array). */
int ccl_add_batch(int dtype, int narr, const long *n, void *const *dst, const void *const *src,
                  void *stream);

/* dst[a] <- src[a] (nbytes[a] bytes, a multiple of 4; 4-byte aligned) for
 * a < narr <= 32, one launch.  No counterpart in the reference: the
 * adjoint's records of forward steps and its per-step inputs. */
int ccl_copy_batch(int narr, const long *nbytes, void *const *dst, const void *const *src,
                   void *stream);

/* Transpose of the deposit post-processing (grid_methods_cl.py:98-151,
 * grid_generic.cl:4-59), in place: row 0 <- row 0 dV_inv[0] - row 1
 * dV_inv[1], row ir <- row ir dV_inv[ir] for ir >= 1. */
int ccl_deposit_postproc_adjoint(int dtype, int M, int nfld, void *const *flds, int Nx, int Nr,
                                 const void *dV_inv, void *stream);

/* Transpose of the ghost rows (grid_methods_cl.py:153-166,
 * grid_generic.cl:63-86), in place: row 1 += (m = 0) or -= (m >= 1)
 * row 0, then row 0 = 0. */
int ccl_warp_axis_adjoint(int dtype, int M, int nfld, void *const *flds, int Nx, void *stream);

/* Transpose of align (particles_methods_cl.py:263-286,
 * particles_generic.cl:156-169): dst[c][sort_indx[i]] = src[c][i] for
 * i < n; entries of dst that no index names are left as they are. */
int ccl_align_adjoint(int dtype, long n, int ncomp, void *const *src, void *const *dst,
                      const uint32_t *sort_indx, void *stream);

/* Transpose of the density profile (particles_methods_cl.py:179-204,
 * particles_generic.cl:6-30) with respect to its knot values: the weights
 * w = w0 f(x) of np particles, f piecewise linear through (xx[k], ff[k]);
 * lff[k] += sum_i lw[i] w[i] / f(x_i) df/dff[k](x_i) (double; 2 <= nloc <=
 * 256 knots, as ccl_dens_profile takes them). */
int ccl_dens_profile_adjoint(int dtype, long np, const void *x, const void *w, const void *lw,
                             const double *xx, const double *ff, const double *dxm1,
                             uint32_t nloc, double *lff, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CHIMERACL_GB300_H */
