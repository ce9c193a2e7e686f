/*
 * mdft_gb300.h -- C ABI of the GB300 (sm_103a) implementation of Mini-MDFT's
 * excess-functional convolution hot path.
 *
 * The entry points replace the reference's C++ operator templates one for
 * one (paths relative to the Mini_MDFT project root):
 *
 *   SpatialGrid + AngularGrid           common/MDFT_Grid.hpp:184-238, :264-469
 *   OrientationProjectionMap            common/MDFT_OrientationProjectionTransform.hpp:55-155
 *   OrientationProjectionTransform      common/MDFT_OrientationProjectionTransform.hpp:217-484
 *   Convolution                         common/MDFT_Convolution.hpp:106-548
 *   IO::LucData (c(q) file reader)      common/IO/MDFT_ReadCLuc.hpp:40-260
 *   get_delta_rho / get_delta_f         common/MDFT_Solvent.hpp:578-660
 *
 * Conventions
 *   - Every array is row-major (Kokkos::LayoutRight).  Complex values are two
 *     interleaved reals (re, im), the layout of Kokkos::complex<T>.
 *   - Orientation fields o: (nx*ny*nz, ntheta, nphi, npsi) real.
 *     Projections p: (np, nx, ny, nz) complex.
 *   - Field pointers are DEVICE pointers on the current CUDA device.  Work is
 *     enqueued on `stream` (a cudaStream_t; NULL = legacy default stream) and
 *     returns without synchronising, like Kokkos kernels on a device
 *     execution space; the caller fences (cudaStreamSynchronize).
 *   - MDFT_F64 handles take double / complex<double> fields (the reference's
 *     ScalarType=double).  MDFT_F32 handles take float / complex<float> fields
 *     (ScalarType=float): the mixed form, whose Wigner/rotation recursions and
 *     grid-wide energy sum stay in FP64.
 *   - No C++ exception crosses this boundary.  Functions return an
 *     mdft_status; mdft_last_error() gives the message of the calling
 *     thread's last failure (the text the reference's Throw_If would raise,
 *     common/MDFT_Asserts.hpp:15-28).
 *   - A handle is not re-entrant: two calls on one handle must not overlap on
 *     the GPU (the reference's OPT shares one o_hat buffer between calls,
 *     common/MDFT_OrientationProjectionTransform.hpp:208-209).
 */
#ifndef MDFT_GB300_H
#define MDFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MDFT_GB300_ABI_VERSION 1

typedef enum {
  MDFT_OK = 0,
  MDFT_ERR_INVALID = 1,     /* bad argument / shape (reference: Throw_If) */
  MDFT_ERR_CUDA = 2,        /* a CUDA runtime call failed */
  MDFT_ERR_IO = 3,          /* c(q) file missing or malformed */
  MDFT_ERR_UNSUPPORTED = 4, /* size outside what the kernels handle */
  MDFT_ERR_NOMEM = 5,       /* device allocation failed */
  MDFT_ERR_TIMEOUT = 6      /* a bounded device wait of an earlier launch on
                               this device ran out: that launch's results are
                               wrong (see mdft_wait_timeouts) */
} mdft_status;

/* MDFT_F64: double fields, FP64 arithmetic (the reference's
 *   ScalarType=double).
 * MDFT_F32: float fields, FP32 arithmetic with FP64 recursions and energy
 *   sum (the mixed form).
 * MDFT_F64_DF: double fields, arithmetic in double-float (each value a pair
 *   of floats, ~48 significand bits, error-free sums and products) on the
 *   FP32 pipes, which on this GPU are 64x wider than the FP64 pipe; results
 *   stay within 1e-12 of the FP64 form.  Recursions (Wigner-d, R(q)) and the
 *   energy sum remain FP64. */
typedef enum { MDFT_F64 = 0, MDFT_F32 = 1, MDFT_F64_DF = 2 } mdft_precision;

typedef struct mdft_grid_s* mdft_grid_t;
typedef struct mdft_opt_s* mdft_opt_t;
typedef struct mdft_conv_s* mdft_conv_t;

int mdft_abi_version(void);
const char* mdft_last_error(void);

/* ---- grids --------------------------------------------------------------
 * SpatialGrid(n_nodes, length) and AngularGrid(mmax, molrotsymorder) in one
 * handle (common/MDFT_Grid.hpp:184-220, :264-398).  Host-only, no GPU work.
 * mmax in [1, 10]; n in [1, 4096] per axis. */
int mdft_grid_create(mdft_grid_t* out, int nx, int ny, int nz, double lx,
                     double ly, double lz, int mmax, int molrotsymorder);
int mdft_grid_destroy(mdft_grid_t g);
/* ints[0..10]: nx ny nz mmax mrso ntheta nphi npsi no np np_new */
int mdft_grid_info(mdft_grid_t g, int* ints);
/* kx,ky,kz (SpatialGrid::kproj, MDFT_Grid.hpp:222-238). */
int mdft_grid_kvectors(mdft_grid_t g, double* kx, double* ky, double* kz);
/* thetaofntheta, wthetaofntheta (ntheta) and w (no), MDFT_Grid.hpp:316-372. */
int mdft_grid_angular(mdft_grid_t g, double* theta, double* wtheta, double* w);
/* OrientationProjectionMap getters p(), m(), mup(), mu(), mu2(),
 * wigner_small_d() (MDFT_OrientationProjectionTransform.hpp:150-155):
 * p (mmax+1, 2mmax+1, mmax/mrso+1), the rest (np), wigner (ntheta, np). */
int mdft_grid_opmap(mdft_grid_t g, int* p, int* m, int* mup, int* mu,
                    int* mu2, double* wigner);
/* The angular transforms at one grid point as dense real matrices (FP64,
 * row-major), the operators the tensor-core path multiplies by: a2p
 * (2 np, no) maps the orientation values to (Re, Im) of the projections
 * (MDFT_OrientationProjectionTransform.hpp:270-380), p2a (no, 2 np) maps
 * them back (:391-484).  Host-only.  No counterpart in the reference. */
int mdft_grid_ang_matrices(mdft_grid_t g, double* a2p, double* p2a);

/* ---- OrientationProjectionTransform ------------------------------------
 * Constructor (MDFT_OrientationProjectionTransform.hpp:217-257): uploads the
 * Wigner-d/quadrature tables to the current device.  With MDFT_ANG_TC=1 in
 * the environment at create time, MDFT_F64_DF and MDFT_F32 handles run
 * angl2proj (except the fused form from xi) and proj2angl as tensor-core
 * GEMMs over the dense per-point matrices (mdft_grid_ang_matrices) with exact
 * BF16 digit slicing, where the shape fits that kernel (at most 288 inputs
 * per point, and the input tile, digit stages and matrix within shared
 * memory: mmax <= 3 for mrso 2); the results agree with the default kernels
 * within each form's tolerance.  Off by default (slower on one GB300 at
 * 64^3 / mmax 3). */
int mdft_opt_create(mdft_opt_t* out, mdft_grid_t g, int precision);
/* Batched plan: one call transforms `batch` same-shape fields stored back to
 * back, o (batch, nx*ny*nz, ntheta, nphi, npsi) and p (np, batch, nx, ny, nz).
 * No counterpart in the reference (one field per call there); it lets a
 * server run many small same-shape jobs as one set of launches.  batch in
 * [1, 65535], batch * nx*ny*nz < 2^31.  mdft_opt_create = batch 1. */
int mdft_opt_create_batched(mdft_opt_t* out, mdft_grid_t g, int precision, int batch);
int mdft_opt_destroy(mdft_opt_t h);
/* angl2proj(o, p), MDFT_OrientationProjectionTransform.hpp:270-380:
 * real o -> complex p. */
int mdft_opt_angl2proj(mdft_opt_t h, const void* o, void* p, void* stream);
/* proj2angl(p, o), MDFT_OrientationProjectionTransform.hpp:391-484:
 * complex p -> real o.  p is read only. */
int mdft_opt_proj2angl(mdft_opt_t h, const void* p, void* o, void* stream);
/* get_delta_rho fused into angl2proj's load: o = rho0 (xi^2 - 1) is formed
 * in registers and never written (MDFT_Solvent.hpp:578-596 followed by
 * MDFT_OrientationProjectionTransform.hpp:270-380). */
int mdft_opt_angl2proj_from_xi(mdft_opt_t h, const void* xi, double rho0,
                               void* p, void* stream);

/* ---- Convolution --------------------------------------------------------
 * Convolution(filename, grid, angular_grid, map, np_luc),
 * MDFT_Convolution.hpp:106-313, from a c(q) table already in memory in the
 * Luc layout: luc_index is 5 x np_luc ints (rows m, n, mu, nu, khi;
 * ReadCLuc.hpp:88-103), luc is (np_luc, nq) complex double (host pointers),
 * dq the q spacing.  nq must be at least int(q_max/dq + 0.5) + 2
 * (ReadCLuc.hpp:65); extra rows are ignored as the reader ignores them.
 * mmax <= 6 (RotationCoeffs, MDFT_Rotation.hpp:29). */
int mdft_conv_create(mdft_conv_t* out, mdft_grid_t g, const int* luc_index,
                     const double* luc, int np_luc, int nq, double dq,
                     int precision);
/* Batched plan (see mdft_opt_create_batched): execute, fft and kspace act on
 * p (np, batch, nx, ny, nz), every field with the same c(q) table.  No
 * counterpart in the reference.  mdft_conv_create = batch 1. */
int mdft_conv_create_batched(mdft_conv_t* out, mdft_grid_t g, const int* luc_index,
                             const double* luc, int np_luc, int nq, double dq,
                             int precision, int batch);
/* Same, reading the Luc text file (ReadCLuc.hpp:40-260). */
int mdft_conv_create_from_file(mdft_conv_t* out, mdft_grid_t g,
                               const char* path, int np_luc, int precision);
int mdft_conv_destroy(mdft_conv_t h);
/* execute(deltarho_p), MDFT_Convolution.hpp:326-548: in place on complex
 * p (np, nx, ny, nz): forward 3-D FFT, per-(q,-q) rotation + OZ + rotation
 * back, inverse 3-D FFT, all unnormalised as in the reference. */
int mdft_conv_execute(mdft_conv_t h, void* p, void* stream);
/* execute(deltarho_p) with its stages timed: events[0..3] are four
 * cudaEvent_t (created by the caller, timing enabled), recorded on `stream`
 * before the forward FFT and after the forward FFT, the k-space step and the
 * inverse FFT.  Same kernels and results as mdft_conv_execute.  No
 * counterpart in the reference (its execute has no stage timers); it exists
 * so that a benchmark can time the stages as execute runs them (the
 * double-float form keeps the projections packed between its stages, which
 * the separate mdft_conv_fft / mdft_conv_kspace calls below do not). */
int mdft_conv_execute_timed(mdft_conv_t h, void* p, void* stream, void* const* events);
/* Same, timed per kernel: events[0..7] are recorded before the forward FFT,
 * after each of its three axis passes (z, y, x), after the k-space step and
 * after each inverse pass (x, y, z).  No counterpart in the reference. */
int mdft_conv_execute_timed_passes(mdft_conv_t h, void* p, void* stream, void* const* events);
/* The two 3-D FFT passes of execute on their own (sign -1 forward,
 * +1 backward; unnormalised), and the k-space step alone. */
int mdft_conv_fft(mdft_conv_t h, void* p, int sign, void* stream);
int mdft_conv_kspace(mdft_conv_t h, void* p, void* stream);
/* Getters gamma_p_map() (npairs x 3 ints), dq(), and sizes
 * (MDFT_Convolution.hpp:316-318). ints: npairs np_new nq */
int mdft_conv_info(mdft_conv_t h, int* ints, double* dq);
int mdft_conv_gamma_p_map(mdft_conv_t h, int* map);
/* mnmunukhi_q() as (np_new, nq) complex double, host copy. */
int mdft_conv_mnmunukhi_q(mdft_conv_t h, double* tab);

/* ---- c(q) files ---------------------------------------------------------------
 * IO::LucData (common/IO/MDFT_ReadCLuc.hpp:40-260) on the host, no GPU work.
 * mdft_luc_read: reads the first int(qmax/dq + 0.5) + 2 q rows of a Luc text
 * file (the rows a grid with that |q_max| needs); with luc_index or luc NULL
 * it only returns nq and dq (call it first to size the arrays).  luc_index is
 * 5 x np_luc ints, luc (np_luc, nq) complex double.
 * mdft_luc_write: writes a table in the layout the reader parses (no
 * counterpart in the reference, which only reads; it lets a producer of
 * c(q) tables hand them to the reference or to this library as files). */
int mdft_luc_read(const char* path, int np_luc, double qmax, int* luc_index, double* luc,
                  int* nq, double* dq);
int mdft_luc_write(const char* path, const int* luc_index, const double* luc, int np_luc,
                   int nq, double dq, const char* header);

/* ---- energy ---------------------------------------------------------------
 * get_delta_rho(exec, xi, delta_rho, rho0), MDFT_Solvent.hpp:578-596:
 * delta_rho[i] = rho0 (xi[i]^2 - 1) over n elements.  precision selects
 * double or float arrays. */
int mdft_get_delta_rho(const void* xi, void* delta_rho, size_t n, double rho0,
                       int precision, void* stream);
/* get_delta_f(exec, xi, vexc, w, delta_f, ff, rho0, prefactor),
 * MDFT_Solvent.hpp:617-660: delta_f = 2 rho0 xi vexc and
 * ff = sum_r rho0 prefactor sum_o vexc w (xi^2 - 1) over xi, vexc, delta_f
 * of shape (nxyz, no) and w (no) (all device pointers, w always double).
 * ff_dev is a device double; it is overwritten (the reference sets ff = 0
 * first).  The sum over points is deterministic on a given GPU (a fixed
 * reduction tree with compensated partial sums; its shape follows the
 * device's SM count and the kernel's occupancy).  Uses a stream-ordered
 * temporary of 16 bytes per 32 points, plus 16, from the library's own pool
 * (mdft_scratch_pool). */
int mdft_get_delta_f(const void* xi, const void* vexc, const double* w,
                     void* delta_f, double* ff_dev, size_t nxyz, int no,
                     double rho0, double prefactor, int precision,
                     void* stream);
/* The stream-ordered memory pool (a cudaMemPool_t) on the current device
 * that the library's allocating entry points take their temporaries from,
 * created at the first use; it keeps up to 64 MiB mapped between calls, so
 * calls made after a synchronize do not map their scratch again.  No
 * counterpart in the reference. */
int mdft_scratch_pool(void** pool);

/* get_delta_f for callers that cannot allocate device memory while they run
 * (an application that gives the whole GPU to its own pool allocator up
 * front and forbids allocations behind its back, or a loop that must not
 * pay for an allocation call).  No counterpart in the reference: it is the
 * same computation as mdft_get_delta_f, but its per-CTA partial sums live in
 * one fixed 1 MiB array of the library's device memory (held on every GPU
 * that loads the library until exit) instead of a stream-ordered temporary;
 * it calls no allocation routine.  Limit: nxyz <= 2,097,152 grid points
 * (128^3); larger grids return MDFT_ERR_UNSUPPORTED.  All calls share the
 * array, so calls that overlap on the GPU race and must be serialised by the
 * caller.  A call on a stream that is not capturing looks the array's
 * address up on the current device (so a context reset by cudaDeviceReset is
 * picked up); a call on a capturing stream reuses the address of the last
 * such lookup on that device, so the first call on a device must come before
 * any stream capture. */
int mdft_get_delta_f_noalloc(const void* xi, const void* vexc, const double* w,
                             void* delta_f, double* ff_dev, size_t nxyz, int no,
                             double rho0, double prefactor, int precision,
                             void* stream);

/* Diagnostics: number of bounded device waits (on the asynchronous copies of
 * the FFT's tensor-memory-access tiles, or on the flags of the server's
 * persistent kernels) that ran out of time on the current device since the
 * library was loaded; such a kernel leaves its output wrong.  Each new
 * timeout also makes the next call that launches that kind of work on the
 * device return MDFT_ERR_TIMEOUT, so callers need not poll this.  No
 * counterpart in the reference. */
int mdft_wait_timeouts(int* count);
/* Diagnostics: exercises the error path of those waits without a fault or a
 * hang -- one CTA waits on a barrier that nothing completes, gives up after
 * `spins` polls (1 <= spins <= 2^20) and records the timeout as a real one;
 * the next FFT launch on the device then returns MDFT_ERR_TIMEOUT.  No
 * counterpart in the reference. */
int mdft_wait_selftest(int spins, void* stream);
/* Diagnostics: the same for the grid barrier of the persistent L-BFGS kernel
 * (the minimiser's and the server's vector passes, one cooperative launch per
 * step): one cooperative launch whose blocks meet at that barrier, which
 * expects `missing` (0..1024) more arrivals than there are blocks.  With
 * missing = 0 it passes; with missing > 0 every block gives up after about a
 * second of polling and the timeout is recorded, so the next call that
 * checks the device's waits returns MDFT_ERR_TIMEOUT.  No counterpart in the
 * reference. */
int mdft_grid_barrier_selftest(int missing, void* stream);

/* ---- job server -----------------------------------------------------------
 * No counterpart in the reference (which evaluates one field per call).  A
 * server takes jobs from any host thread and runs them on the device that was
 * current at create, on its own worker thread:
 *   - a job is one field xi (nx*ny*nz, ntheta, nphi, npsi) on one grid with
 *     one registered solvent; each of its n_steps steps evaluates the cproj
 *     excess energy and gradient at xi (get_delta_rho, angl2proj,
 *     Convolution::execute, proj2angl, get_delta_f: src/mini-mdft.hpp:137-183)
 *     and moves xi by -step * gradient;
 *   - jobs with the same solvent and grid advance together with batched
 *     launches (up to max_batch per group), replayed from CUDA graphs;
 *   - groups are created only within hbm_budget_bytes of device memory
 *     (0: 80 % of the free memory at create); jobs wait until theirs fits.
 * Fields are host arrays in the server's precision (double for MDFT_F64 and
 * MDFT_F64_DF, float for MDFT_F32). */
typedef struct mdft_server_s* mdft_server_t;
int mdft_server_create(mdft_server_t* out, int precision, int max_batch, size_t hbm_budget_bytes);
/* Fails every unfinished job, waits for the worker, frees the device memory. */
int mdft_server_destroy(mdft_server_t s);
/* A solvent: its angular grid (mmax <= 6), c(q) table as for
 * mdft_conv_create, bulk density rho0 and the energy prefactor of
 * get_delta_f. */
int mdft_server_add_solvent(mdft_server_t s, int mmax, int mrso, const int* luc_index,
                            const double* luc, int np_luc, int nq, double dq,
                            double rho0, double prefactor, int* solvent_id);
/* Queues a job (xi0 is copied; n_steps <= 4096) and returns at once. */
int mdft_server_submit(mdft_server_t s, int solvent_id, int nx, int ny, int nz, double lx,
                       double ly, double lz, const void* xi0, int n_steps, double step,
                       long long* job_id);
/* Blocks until the job is done, then hands over its final xi (host, may be
 * NULL), the energy of every step (n_steps doubles, may be NULL) and its
 * latency from submit (seconds, may be NULL).  Each job is waited for once. */
int mdft_server_wait(mdft_server_t s, long long job_id, void* xi_out, double* ff_out,
                     double* latency_s);
/* Solute jobs (no counterpart in the reference): each job carries a solute
 * and is minimised with the full functional of mdft_solver_minimize (L-BFGS
 * on E_id + E_ext + E_exc, every precision's xi in double), its minimiser
 * state resident on the device; same-shape jobs share one batched energy
 * evaluation per step.  The solvent's molecular model first: sites as for
 * mdft_vext_lj_coulomb (molecular frame), kT [kJ/mol], vmax [kJ/mol]. */
int mdft_server_set_solvent_model(mdft_server_t s, int solvent_id, const double* sites, int n_sites, double kT,
                                  double vmax);
/* Queues a solute job (sites in box coordinates, copied; xi0: host doubles,
 * (nx*ny*nz, no), NULL for xi = 1) that runs until max |dE/dxi| <= gtol, no
 * step lowers E, or max_iter iterations. */
int mdft_server_submit_solute(mdft_server_t s, int solvent_id, int nx, int ny, int nz, double lx, double ly,
                              double lz, const double* solute_sites, int n_sites, const double* xi0, int max_iter,
                              double gtol, long long* job_id);
/* Blocks until the solute job is done: final xi (host doubles, may be NULL),
 * trace ((max_iter + 1) rows of E_total, E_id, E_ext, E_exc, max |dE/dxi|,
 * may be NULL), iterations, status (0 gtol reached, 1 E flat, 2 max_iter,
 * 3 no decrease along the direction) and latency (each may be NULL). */
int mdft_server_wait_solute(mdft_server_t s, long long job_id, double* xi_out, double* trace_out, int* iterations,
                            int* status, double* latency_s);
/* out[0..7]: jobs done, jobs done per second since the first submit, p50 and
 * p99 latency (s), job groups held, peak device bytes of the groups, group
 * steps replayed from captured graphs, group steps launched directly. */
int mdft_server_stats(mdft_server_t s, double* out);

/* ---- Solute external potential and the minimiser --------------------------
 * The loop around Solver::energy_cproj_mrso (src/mini-mdft.hpp:130-183): the
 * reference defines its data -- solvent and solute sites
 * (common/MDFT_Solvent.hpp:410-494, common/MDFT_Solute.hpp:150-200), the
 * orientation rotation matrices (common/MDFT_Grid.hpp:283-310), qfact
 * (common/MDFT_Constants.hpp:46-47) -- but computes neither vext nor a
 * minimiser step; these entry points do, with the formulas of
 * mini_mdft_gb300/csrc/solver.cu.
 *
 * Sites are rows (q [e], sigma [A], epsilon [kJ/mol], x, y, z [A]): solvent
 * sites in the molecular frame (the reference's Solvent tables), solute sites
 * in box coordinates.  vext (device, (nx*ny*nz, no) doubles, the layout of
 * xi) = LJ 12-6 (Lorentz-Berthelot) + qfact q_a q_s / d between every
 * solvent site of each orientation and every solute site, minimum image,
 * clamped to [-vmax, vmax] kJ/mol.  Returns when vext is written. */
int mdft_vext_lj_coulomb(mdft_grid_t grid, const double* solvent_sites, int n_solvent_sites,
                         const double* solute_sites, int n_solute_sites, double vmax,
                         double* vext, void* stream);

/* An L-BFGS minimiser of E(xi) = E_id + E_ext + E_exc on one field (batch-1
 * handles of one grid and precision; xi, vext and the gradient are FP64 in
 * every precision, the cproj step runs in the handles' precision).  vext
 * (device, copied; NULL: no external potential), kT [kJ/mol], rho0 and the
 * get_delta_f prefactor, history: stored curvature pairs (1..32). */
typedef struct mdft_solver_s* mdft_solver_t;
int mdft_solver_create(mdft_solver_t* out, mdft_opt_t opt, mdft_conv_t conv, const double* vext,
                       double kT, double rho0, double prefactor, int history);
/* E and dE/dxi at xi (device): grad (device, may be NULL), terms (host, 5):
 * E_total, E_id, E_ext, E_exc, max |dE/dxi|.  Returns when terms are set. */
int mdft_solver_energy(mdft_solver_t s, const double* xi, double* grad, double* terms, void* stream);
/* Minimises from xi (device, overwritten with the last accepted iterate)
 * until max |dE/dxi| <= gtol, |Delta E| <= ftol max(1, |E|), no step along
 * the search direction lowers E, or max_iter iterations.  trace (host, may be
 * NULL): (max_iter + 1) rows of the 5 terms, row 0 at the start, row i after
 * iteration i; iterations (may be NULL): iterations taken. */
int mdft_solver_minimize(mdft_solver_t s, double* xi, int max_iter, double gtol, double ftol,
                         double* trace, int* iterations, void* stream);
/* How the last mdft_solver_minimize ended: 0 max |dE/dxi| <= gtol, 1 |Delta E|
 * <= ftol max(1, |E|), 2 max_iter reached, 3 no step along the search
 * direction lowered E (after 40 halvings), -1 never run. */
int mdft_solver_status(mdft_solver_t s, int* status);
int mdft_solver_destroy(mdft_solver_t s);

#ifdef __cplusplus
}
#endif
#endif /* MDFT_GB300_H */
