/*
 * wannier90_gb300.h -- C ABI of the GB300 MLWF (wann_main) engine.
 *
 * The first group of entry points carries the names, argument order and meaning of
 * Wannier90's own C binding of its library (src/c_interface.F90, prototypes in
 * src/wannier90.hh), so a code that drives Wannier90 through `w90_create`/`cset_*`/
 * `cinput_setopt`/`cwannierise`/`cget_*` can link this library instead for the
 * wannierisation step.  Differences, all at the type level:
 *   - keywords and seednames are NUL-terminated `const char*` (the reference passes a
 *     Fortran CFI descriptor built by the std::string helpers of wannier90.hh; the
 *     same helper overloads are provided below for C++ callers);
 *   - `int&` out-arguments are `int*` (identical calling convention);
 *   - complex arrays are `double*` pointing at interleaved (re, im) pairs, i.e. the
 *     memory of `std::complex<double>` / Fortran `complex(8)` arrays;
 *   - the MPI communicator argument of cinput_setopt is accepted and ignored (one
 *     process drives one GPU; k-points are never distributed).
 *
 * Array layouts are the reference's (Fortran column-major):
 *   m matrix   [nk][nntot][nb][nb]   element (m,n,b,k) at m + nb*(n + nb*(b + nntot*k))
 *   u matrix   [nk][nw][nw]          element (m,n,k)  at m + nw*(n + nw*k)
 *   u_opt      [nk][nw][nb]
 *   eigval     [nk][nb]
 *   nnkp       [nntot][nk] int32, 1-based k+b indices (cget_nnkp)
 *   centres    [nw][3], spreads [nw]
 * Error convention (src/error.F90:25-35): ierr = 0 ok; >0 error (1 fatal, 2 alloc,
 * 5 input/unsupported option, 6 file); <0 warning (-1 not converged).
 *
 * The engine never aborts the process; CUDA errors map to ierr = 1, device OOM to 2.
 */
#ifndef WANNIER90_GB300_H
#define WANNIER90_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- handle lifecycle: src/c_interface.F90:10-25 ------------------------------- */
void* w90_create(void);
void w90_delete(void* handle);

/* ---- options: src/c_interface.F90:179-247 (cset_option_*), library keywords of
 *      w90_set_option (src/library_interface.F90:667-808) ---------------------------- */
void cset_option_int(void* handle, const char* keyword, int value);
void cset_option_int3(void* handle, const char* keyword, const int* value3);
void cset_option_intx(void* handle, const char* keyword, const int* values, int count);
void cset_option_float(void* handle, const char* keyword, double value);
/* value: double[3][3] row-major, row i = a_i (Angstrom) for unit_cell_cart */
void cset_option_float33(void* handle, const char* keyword, const double* value33);
/* value: double[x][y] row-major (e.g. kpoints: x = num_kpts, y = 3) */
void cset_option_floatxy(void* handle, const char* keyword, const double* values, int x, int y);

/* ---- process options, build the k-mesh: src/c_interface.F90:49-68 ----------------
 * Keywords read by the engine besides the system ones: num_iter, num_cg_steps, conv_tol,
 * conv_window, trial_step / fixed_step, precond (+ mp_grid), guiding_centres,
 * num_no_guide_iter, num_guide_cycles, slwf_num, slwf_constrain, slwf_lambda,
 * site_symmetry, symmetrize_eps, dis_*,
 * search_shells, kmesh_tol, iprint.  Block data the C binding cannot pass as text comes
 * as floatxy tables: guiding_centres_frac (num_wann x 3, the projection sites) and
 * slwf_centres_frac (num_wann x 3, the constrained centres: the <slwf_centres> rows
 * over the projection sites; without it slwf_constrain uses guiding_centres_frac).
 * site_symmetry (+ symmetrize_eps) needs w90g_set_sitesym;
 * gamma_only, conv_noise_amp > 0 and dis_spheres_num > 0 give ierr 5. */
void cinput_setopt(void* handle, const char* seedname, int* ierr, int comm);

/* ---- .win input: cinput_reader, src/c_interface.F90:70-80 (w90_input_reader,
 *      src/library_interface.F90:294-360) --------------------------------------------
 * After cinput_setopt: reads seedname.win (the seedname given to cinput_setopt) with the
 * reference's tokenizer rules (lower case, '!' and '#' comments, `key = value`,
 * `key : value` or `key value`, begin/end blocks); a keyword outside the set wannier90.x
 * and postw90.x accept (src/readwrite.F90:903-1176, plus the engine's gpu_* keys), or one
 * given twice, gives ierr 5 with the reference's message.  Keywords of the .win take
 * precedence over earlier options; the system (num_wann, num_bands, mp_grid,
 * unit_cell_cart, kpoints) must agree with cinput_setopt's (else 5); the setup is then
 * redone with the merged options.  Called before cinput_setopt or with options set
 * since: ierr 1.  File missing: 6. */
void cinput_reader(void* handle, int* ierr);
/* cinput_reader_special (src/wannier90.hh:11, declared there without a definition in
 * src/c_interface.F90): the whole input, system included, from seedname.win -- the file
 * form of cset_option_* + cinput_setopt.  unit_cell_cart may give `bohr` or `ang` units;
 * projection-derived tables (guiding_centres_frac, slwf_centres_frac) still come through
 * cset_option_floatxy.  ierr as cinput_setopt / cinput_reader. */
void cinput_reader_special(void* handle, const char* seedname, int* ierr);

/* ---- data pointers (caller keeps ownership): src/c_interface.F90:82-127 ----------- */
void cset_eigval(void* handle, double* eigval);
void cset_m_local(void* handle, double* m_matrix);
void cset_u_matrix(void* handle, double* u_matrix);
void cset_u_opt(void* handle, double* u_opt);

/* cset_a_matrix (src/wannier90.hh:31): the caller's projections A_mn(k), complex
 * [nk][nw][nb].  coverlaps reads seedname.amn into it; cproject_overlap (nb = nw) and
 * cdisentangle copy it into u_matrix / u_opt before they start. */
void cset_a_matrix(void* handle, double* a_matrix);
/* cset_kpoint_distribution (src/wannier90.hh:28; set_kpoint_distribution,
 * src/wannier_prog.F90:798-820): dist[nk] = the rank owning each k-point.  The engine is
 * one process on one GPU: the all-zero distribution is accepted, any other makes the next
 * work call (coverlaps, cproject_overlap, cdisentangle, cwannierise) return 5. */
void cset_kpoint_distribution(void* handle, const int* dist);
/* cset_parallel_comms (src/wannier90.hh:29): the MPI communicator (Fortran handle);
 * stored, not used (no collective runs: every k-point is on this GPU). */
void cset_parallel_comms(void* handle, int comm);
/* coverlaps (src/wannier90.hh:21; overlaps, src/wannier_prog.F90:478-537): reads
 * seedname.mmn into m_local and seedname.amn into the projections -- the cset_a_matrix
 * buffer if set, else u_matrix (nb = nw) or u_opt (nb > nw) -- with overlap_read's checks
 * and messages (src/overlap.F90:234-366).  ierr: 1 when called before cinput_setopt or a
 * buffer is missing, 6 for a file error. */
void coverlaps(void* handle, int* ierr);
/* cchkpt (src/wannier90.hh:9; write_chkpt, src/wannier_prog.F90:575-700): writes
 * seedname.chk, checkpoint label `label` ("postdis", "postwann"), in the unformatted
 * layout of w90_wannier90_readwrite_write_chkpt (src/wannier90_readwrite.F90:2278-2373):
 * exclude_bands, lattice, k-points, u_matrix, u_opt, the leading nw x nw block of every
 * m_local block, centres and spreads of the last wannierisation, and after a
 * disentanglement Omega_I, lwindow and ndimwin.  No ierr (as the prototype): failures
 * (missing buffers, file errors) are reported by w90g_last_error. */
void cchkpt(void* handle, const char* label);

/* ---- work: src/c_interface.F90:38-47 (cwannierise -> w90_wannierise ->
 *      wann_main, src/library_interface.F90:464-530) ----------------------------------
 * On entry m holds the projected M^(0) and u the initial U (after cproject_overlap);
 * on exit u holds the final U and m is rotated in place to the final gauge. */
void cwannierise(void* handle, int* ierr);

/* ---- disentanglement: src/c_interface.F90:27-36 (cdisentangle -> w90_disentangle ->
 *      dis_main + setup_m_loc, src/library_interface.F90:362-420; prototype
 *      src/wannier90.hh:22) ---------------------------------------------------------------
 * On entry m holds the raw overlaps (nb x nb blocks), u_opt the projections A (nb x nw)
 * and eigval the band energies; the dis_* keywords of cinput_setopt set the windows and
 * the Omega_I iteration.  On exit u_opt holds the optimal subspace (outer-window rows,
 * from the first), u the internal_find_u rotation (nw x nw), and the top-left nw x nw of
 * every m block U^dagger U_opt^dagger M U_opt(k+b) U(k+b) -- the input of cwannierise,
 * which then reads and writes those sub-blocks.  Needs nw <= nb <= 64. */
void cdisentangle(void* handle, int* ierr);

/* ---- getters: src/c_interface.F90:129-177 ------------------------------------------ */
void cget_nn(void* handle, int* nntot);
void cget_nnkp(void* handle, int* nnkp);
void cget_centres(void* handle, double* centres);
void cget_spreads(void* handle, double* spreads);

/* ---- additions the isolated-band C path needs -----------------------------------
 * cproject_overlap: Loewdin initialisation w90_project_overlap -> overlap_project
 *   (src/library_interface.F90:422-462, src/overlap.F90:758-952), which the reference
 *   exports to Fortran only.  On entry u holds A(k) (num_wann x num_wann), m the raw
 *   overlaps; on exit u = Z V^dagger and m = U^dagger M U(k+b).
 * cget_omega: (Omega_I, Omega_D, Omega_OD, Omega_total) of the last wannierisation
 *   (common_data%omega / wann_spread, src/wannierise.F90:457-470).  With selective
 *   localisation (slwf_num < num_wann) Omega_I is left as it was (the disentanglement's,
 *   else 0), Omega_D is (1 - lambda) times the objective WFs' part and the third entry is
 *   Omega_IOD + Omega_nu, what the reference prints as O_IOD. */
void cproject_overlap(void* handle, int* ierr);
void cget_omega(void* handle, double* omega4);
/* cget_gkpb: nncell of kmesh_info ([nntot][nk][3] int32), the G offsets of k+b
 *   (w90_get_gkpb, src/library_interface.F90:866-900) */
void cget_gkpb(void* handle, int* gkpb);

/* ---- engine extensions (no counterpart in the reference) ---------------------------- */
/* Last error message ("" when none). */
const char* w90g_last_error(void* handle);
/* Per-iteration record of the last wannierisation: rows of 10 doubles
 *   (iter, delta Omega, RMS gradient, Omega_total, Omega_D, Omega_OD, lquad, alphamin,
 *    device timestamp ns, Omega_nu) for iter = 0 (initial state) .. niter; with
 *   selective localisation Omega_OD holds Omega_IOD + Omega_nu and Omega_nu the centre
 *   constraint's term (0 otherwise).
 * Returns the number of rows written (<= max_rows). */
int w90g_get_log(void* handle, double* rows, int max_rows);
/* Disentanglement record of the last cdisentangle: rows of 5 doubles
 *   (iter, Omega_I(i-1), Omega_I(i), delta (frac.), seconds) -- the "<-- DIS" lines of
 *   dis_extract (src/disentangle.F90:2480-2490).  Returns the rows written. */
int w90g_get_dis_log(void* handle, double* rows, int max_rows);
/* Outer window of the last cdisentangle per k: ndimwin[nk] states from band nfirstwin[nk]
 * (0-based) -- dis_manifold%ndimwin / nfirstwin, and lwindow(i,k) = nfirstwin <= i <
 * nfirstwin + ndimwin, as the checkpoint stores them. */
void w90g_get_dis_windows(void* handle, int* ndimwin, int* nfirstwin);
/* Symmetry data of the symmetry-adapted mode (site_symmetry = T; what sitesym_read reads
 * from the .dmn file, src/sitesym.F90:698-765; the reference's C binding has no way to
 * pass it): the file's counts nb, nsym, nkirr, nk; 1-based ik2ir[nk], ir2ik[nkirr],
 * kptsym(nsym, nkirr); d_matrix_wann(nw, nw, nsym, nkirr) and d_matrix_band(nb, nb, nsym,
 * nkirr), Fortran order, complex as (re, im) pairs.  After cinput_setopt.  Returns the
 * ierr: 6 when the counts or indices disagree with the handle (the reference's
 * "Number of bands / k-points is not correct" messages), 1 when the stars do not cover
 * the mesh.  With site_symmetry = T, cproject_overlap makes the initial U symmetry-
 * adapted, cdisentangle runs the symmetry-adapted disentanglement (outer window only, as
 * in the reference) and cwannierise symmetrises the gradient and rotations. */
int w90g_set_sitesym(void* handle, int nb, int nsym, int nkirr, int nk, const int* ik2ir, const int* ir2ik,
                     const int* kptsym, const double* d_wann, const double* d_band);
/* (final Omega_I = omega%invariant, converged 0/1, iterations, most Jacobi sweeps of a
 *  Z eigenproblem) of the last cdisentangle */
void w90g_get_dis_info(void* handle, double* info4);
/* cdisentangle on DEVICE buffers (same layouts; d_eig (nb, nk) is read back to the host
 * for the windows).  Outputs are written back on the device; w90g_wannierise_device on
 * the same d_m / d_u then works on the top-left nw x nw blocks. */
void w90g_disentangle_device(void* handle, double* d_m_matrix, double* d_u_opt, double* d_u_matrix,
                             const double* d_eigval, int* ierr);
/* Same, timing every kernel launch with CUDA events: ms[i] / counts[i] per kernel i
 * (names from w90g_dis_kernel_name, "" past the last kernel).  Returns ierr. */
int w90g_profile_dis_device(void* handle, double* d_m_matrix, double* d_u_opt, double* d_u_matrix,
                            const double* d_eigval, double* ms, int* counts);
const char* w90g_dis_kernel_name(int i);
/* centres/spreads per iteration: rows of 4*num_wann doubles (x[W], y[W], z[W], spread[W]) */
int w90g_get_log_centres(void* handle, double* rows, int max_rows);
/* Same as cwannierise / cproject_overlap but m and u are DEVICE pointers (CUDA memory of
 * the current device, same layouts); results are written back to them on the device. */
void w90g_wannierise_device(void* handle, double* d_m_matrix, double* d_u_matrix, int* ierr);
void w90g_project_overlap_device(void* handle, double* d_m_matrix, double* d_u_matrix, int* ierr);
/* Batched form: nprob independent problems, each set up on its own handle
 * (cinput_setopt), with device buffers d_m[i], d_u[i] (layouts as above), solved together:
 * problems are grouped by M-update variant (tensor path at padded width 8/16/32/64/128 when
 * the handle sets gpu_tensor, FP64 path otherwise); each group runs as one
 * engine whose captured iteration covers all its problems, groups run concurrently on
 * their own streams.  Per-problem status in ierr[i]; results via the handles' getters.
 * No counterpart in the reference (which solves one problem per library call). */
void w90g_wannierise_batch_device(void** handles, int nprob, double** d_m, double** d_u, int* ierr);
/* Run the engine's work on a caller-provided cudaStream_t (NULL = the engine's own). */
void w90g_set_stream(void* handle, void* cuda_stream);
/* ---- seed files: overlap_read (src/overlap.F90:234-366) and the .eig reader
 *      (src/readwrite.F90:583-635), parsed in parallel on the host ------------------------
 * m: complex (nb, nb, nntot, nk); each block (k, k2, G) of the file is placed at the slot nn
 * with nnlist[k][nn] = k2 (0-based) and nncell[k][nn][0..2] = G, as cget_nnkp / cget_gkpb
 * give them.  a: complex (nb, nproj, nk).  eig: (nb, nk).  nthreads 0 = all cores.
 * Return 0, or 6 (file error) with the reference's message in err (errlen bytes). */
int w90g_read_mmn(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell,
                  double* m_matrix, int nthreads, char* err, int errlen);
int w90g_read_amn(const char* path, int nb, int nproj, int nk, double* a_matrix, int nthreads, char* err,
                  int errlen);
int w90g_read_eig(const char* path, int nb, int nk, double* eigval, char* err, int errlen);
/* .mmn straight into DEVICE memory d_m_matrix (same layout), parsed on the GPU on the
 * caller's stream (NULL = default stream): records indexed and numbers converted by
 * kernels (Clinger's exact fast path); a file outside that path (more than 19 digits or
 * 2^53 in a mantissa, exponents beyond 10^+-22, blank records, two blocks for one slot)
 * is read by w90g_read_mmn and copied, with the same result.  *used_gpu: 1 if the
 * kernels parsed it; *launches: kernels launched; timing3 (NULL or 3 doubles): ms of the
 * value-conversion kernel, of all parse kernels, of the text copy.  Return as
 * w90g_read_mmn. */
int w90g_read_mmn_device(const char* path, int nb, int nk, int nntot, const int* nnlist, const int* nncell,
                         double* d_m_matrix, void* cuda_stream, int* used_gpu, long long* launches,
                         double* timing3, char* err, int errlen);
/* Kernels launched by the last wannierisation plus the last disentanglement on this handle. */
long long w90g_kernel_launches(void* handle);
/* Profiling run of wannierise on device buffers: every kernel launched alone and timed
 * with CUDA events on the launching stream (at most max_iters iterations).  ms[i] and
 * counts[i] (w90g_profile_kernel_name(i), i < 8) receive total time and launches that
 * did work.  Returns ierr.  The per-kernel sequence and arithmetic equal cwannierise's. */
int w90g_profile_device(void* handle, double* d_m_matrix, double* d_u_matrix, int max_iters,
                        double* ms, int* counts);
const char* w90g_profile_kernel_name(int i);
/* W^3 complex products spent by exp(s D) and U dU during the last profiling run (the
 * per-matrix Taylor degree and squarings are data dependent). */
double w90g_profile_exp_products(void* handle);
/* FP64 FMA throughput of the current device in TFLOP/s (dependent-chain probe). */
double w90g_measure_fp64_peak(void);
/* ---- Serving loop (continuous batching).  No counterpart in the reference, which solves
 * one problem per library call (w90_wannierise, src/library_interface.F90:464-530).
 * A server admits queued jobs first-in first-out while the device bytes of its running
 * jobs stay within hbm_budget_bytes and fewer than max_active jobs run; running jobs
 * overlap on the GPU (one stream each), are polled every chunk_iters iterations, and
 * free their memory and slot when they converge.  Each job is solved exactly as by
 * w90g_wannierise_device on the same handle (same kernels, bitwise the same result).
 * Thread safety: submit/poll/pending/drain may be called from any thread; a submitted
 * handle and its buffers belong to the server until the job's tag has been polled. */
void* w90g_server_create(double hbm_budget_bytes, int max_active, int chunk_iters);
/* d_m / d_u: device buffers holding the projected M0 (m_matrix layout) and U0, written
 * before the call (the caller's stream synchronised); the final M and U are written back
 * to them.  Returns 0 (queued), 2 when the job alone exceeds the budget, 1/5 on bad input. */
int w90g_server_submit(void* server, void* handle, double* d_m, double* d_u, long long tag);
/* Collect up to max completed jobs: tag, ierr (as w90g_wannierise_device), and the
 * submit / admission / completion times in seconds on the server's clock.  Returns the count. */
int w90g_server_poll(void* server, long long* tags, int* ierr, double* t_submit, double* t_admit,
                     double* t_done, int max);
int w90g_server_pending(void* server);          /* queued + running jobs */
void w90g_server_drain(void* server);           /* block until no job is queued or running */
/* peak running jobs, peak admitted bytes, jobs completed, iterations completed */
void w90g_server_stats(void* server, double* out4);
double w90g_server_now(void* server);           /* the server's clock (s since creation) */
void w90g_server_delete(void* server);          /* finishes the queued and running jobs first */
/* Wigner-Seitz points of the Born-von Karman supercell used by the preconditioner
 * (replaces hamiltonian_wigner_seitz, src/hamiltonian.F90:689-853, as called from
 * hamiltonian_setup for wann_main, src/wannierise.F90:269-274).  Host only.
 * real_lattice33: rows a_1..a_3 (Angstrom); search_size3: ws_search_size (default 2);
 * irvec_out [max_pts][3], ndegen_out [max_pts].  Returns nrpts (> max_pts: only the count
 * is returned), or -1 when the sum rule fails. */
int w90g_ws_vectors(const double* real_lattice33, const int* mp_grid3, const int* search_size3,
                    double ws_distance_tol, int* irvec_out, int* ndegen_out, int max_pts);
/* Loewdin projection (as w90g_project_overlap_device) that allocates no device memory.
 * No counterpart in the reference.  For callers that cannot call cudaMalloc where they
 * project: e.g. a DFT code whose device memory all belongs to its own pool allocator.
 * d_m_matrix / d_u_matrix are the caller's device buffers (layouts as above; u holds
 * A(k) on entry), updated in place; nnkp is the host array cget_nnkp returns
 * ([nntot][num_kpts], 1-based).  Scratch lives in a file-scope device array of about
 * 4.3 MB that every GPU loading the library keeps until exit; limits num_wann <= 32,
 * num_kpts <= 4096, num_kpts*nntot <= 8192, and every nnkp entry in 1..num_kpts
 * (anything else returns 5 without GPU work).  Every call resolves that array's address
 * (cudaGetSymbolAddress); the first call on a device, and the first after a device
 * reset, also sets kernel attributes, so make it before any stream capture.  Calls share
 * the array: calls whose GPU work overlaps (other streams or threads) race.  An error
 * already pending on the calling thread (cudaPeekAtLastError) makes the call return 1
 * and is left pending.  cuda_stream may be NULL (legacy default stream).  Returns 0 ok,
 * 1 CUDA error / rank-deficient A(k), 5 sizes or nnkp out of range.  Synchronises the
 * stream before returning. */
int w90g_project_overlap_noalloc(int num_wann, int num_kpts, int nntot, const int* nnkp,
                                 double* d_m_matrix, double* d_u_matrix, void* cuda_stream);

#ifdef __cplusplus
}  /* extern "C" */

#include <complex>
#include <string>
/* std::string helpers with the reference's names and argument lists (src/wannier90.hh:43-99) */
inline void cinput_setopt(void* blob, std::string seed, int& ierr, int comm = 0) {
  cinput_setopt(blob, seed.c_str(), &ierr, comm);
}
inline void cset_option(void* blob, std::string key, int x) { cset_option_int(blob, key.c_str(), x); }
inline void cset_option(void* blob, std::string key, int x[3]) { cset_option_int3(blob, key.c_str(), x); }
inline void cset_option(void* blob, std::string key, int* x, int y) { cset_option_intx(blob, key.c_str(), x, y); }
inline void cset_option(void* blob, std::string key, double x[][3]) {
  cset_option_float33(blob, key.c_str(), &x[0][0]);
}
inline void cset_option(void* blob, std::string key, double x) { cset_option_float(blob, key.c_str(), x); }
inline void cset_option(void* blob, std::string key, double* x, int i1, int i2) {
  cset_option_floatxy(blob, key.c_str(), x, i1, i2);
}
inline void cinput_reader(void* blob, int& ierr) { cinput_reader(blob, &ierr); }
inline void cinput_reader_special(void* blob, std::string seed, int& ierr) {
  cinput_reader_special(blob, seed.c_str(), &ierr);
}
inline void cchkpt(void* blob, std::string label) { cchkpt(blob, label.c_str()); }
inline void coverlaps(void* blob, int& ierr) { coverlaps(blob, &ierr); }
inline void cset_a_matrix(void* blob, std::complex<double>* a) { cset_a_matrix(blob, reinterpret_cast<double*>(a)); }
inline void cdisentangle(void* blob, int& ierr) { cdisentangle(blob, &ierr); }
inline void cwannierise(void* blob, int& ierr) { cwannierise(blob, &ierr); }
inline void cproject_overlap(void* blob, int& ierr) { cproject_overlap(blob, &ierr); }
inline void cget_nn(void* blob, int& n) { cget_nn(blob, &n); }
inline void cset_m_local(void* blob, std::complex<double>* m) { cset_m_local(blob, reinterpret_cast<double*>(m)); }
inline void cset_u_matrix(void* blob, std::complex<double>* u) { cset_u_matrix(blob, reinterpret_cast<double*>(u)); }
inline void cset_u_opt(void* blob, std::complex<double>* u) { cset_u_opt(blob, reinterpret_cast<double*>(u)); }
#endif

#endif /* WANNIER90_GB300_H */
