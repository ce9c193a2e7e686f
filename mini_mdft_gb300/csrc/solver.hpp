// solver.hpp -- the minimiser's device work and its per-field state, shared
// by the single-field solver (solver.cu, mdft_solver_*) and the job server
// (server.cu), which advances many fields' minimisers with one batched
// energy evaluation per step.
#pragma once
#include <vector>

#include "common.cuh"

namespace mdft {

// Constants of the xi functional (formulas in solver.cu).
struct EgConst {
  double kT, rho0, dv, prefactor;
};

// The solute's external potential on every grid point and orientation of g,
// written to vext (device, (N, no) doubles); returns when it is written.
void vext_compute(const Grid& g, const double* solvent_sites, int n_solvent, const double* solute_sites,
                  int n_solute, double vmax, double* vext, cudaStream_t s);

// E and dE/dxi at xi: gradient to grad, [E_total, E_id, E_ext, E_exc,
// max |g|] to out (device), and (hinv not null) the inverse of the local
// terms' curvature, floored, as the minimiser's diagonal preconditioner.  vexc is double, or float when vexc_f32; vext
// may be null.  scratch: reduction scratch (reduction_scratch_bytes, zeroed
// once, left zeroed).  nf > 1: nf fields in one launch, field f's arrays at
// f n elements, its out block at f out_stride doubles, its scratch at f
// reduction_scratch_bytes() bytes; each field's sums are the ones it gets
// alone.  dir (FP32, may be null): also out[5] = grad . dir, the slope of E
// along the search direction at xi.
void energy_grad(const EgConst& c, const double* xi, const void* vexc, bool vexc_f32, const double* vext,
                 const double* w, double* grad, long long n, int no, double* out, void* scratch, float* hinv,
                 cudaStream_t s, int nf = 1, long long out_stride = 0, const float* dir = nullptr);
size_t reduction_scratch_bytes();

// xi (double) -> float copy of n values
void to_float(float* y, const double* x, long long n, cudaStream_t s);

// One vector operation of a field's L-BFGS step (built on the host by
// Lbfgs::on_eval, run for every field of a batch by lbfgs_run):
//   kOpPass: x <- [hs h] (a x + c u), then S[out] = scale (v . x), with
//     a = (ja >= 0 ? S[ja] : a0), c = c0 + c1 S[i1] + c2 S[i2] (slots < 0 left
//     out), hs = (jh >= 0 ? S[jh] : 1), scale = (js1 >= 0 ? S[js1] : sc0)
//     (js2 >= 0 ? S[js2] : 1); u and v are FP64 (u64, v64) or FP32 vectors;
//   kOpPair: the curvature pair s = t d, y = gt - g (FP32, into f0 / f1),
//     S[out] = s . y, S[out + 1] = y . h y, S[i1] = rho, S[i2] = gamma (when
//     s . y > 1e-12 y . h y, else rho = 0), and the accepted point kept
//     (x <- xt, g <- gt);
//   kOpCopy: x <- xt, g <- gt;
//   kOpStep: xt <- x + t d.
enum { kOpPass = 0, kOpPair = 1, kOpCopy = 2, kOpStep = 3 };
struct LbOp {
  int type, ja, i1, i2, js1, js2, out, jh, u64, v64;
  double a0, c0, c1, c2, sc0, t;
  float* f0;
  float* f1;
  const void* u;
  const void* v;
  const float* h;
};

// Device state of a batch launch: the partial sums and the grid barrier.
class Lbfgs;
struct LbRunner {
  DevBuf buf;   // partial sums, then the barrier words (count, generation, abort)
  DevBuf prog;  // round form: the op program in device memory
  int blocks = 0;
  // false: one persistent cooperative launch per run (the bounded grid
  // barrier between rounds); true: one ordinary launch per round, for callers
  // whose launches share the GPU with other streams' work (a cooperative
  // launch waits until every SM has room for its CTAs).  Same sums, same
  // order: both forms give identical results.
  bool rounds = false;
  void init();  // on the current device, outside stream capture
};
// Runs the queued operations of k fields' minimisers (on_eval since their
// last run) in one persistent, cooperatively launched kernel: every field's
// operations in order, grid-wide sums between them behind a bounded grid
// barrier.  Each field's sums follow a fixed partition of its elements, so a
// field gets the same results alone and in any batch.  A barrier that runs
// out counts as a timed-out device wait (check_device_waits).
void lbfgs_run(Lbfgs* const* lbs, int k, LbRunner& r, cudaStream_t s);
// One cooperative launch whose blocks meet at the batch kernel's grid
// barrier, expecting `missing` more arrivals than there are blocks: with
// missing > 0 the barrier runs out and is recorded as a timed-out wait.
void grid_barrier_selftest(int missing, LbRunner& r, cudaStream_t s);

// L-BFGS (two-loop recursion with a diagonal initial inverse Hessian, the
// inverse local curvature; Armijo backtracking) of one field.  The host
// keeps only the line-search bookkeeping; every scalar of the recursion
// (alpha_i, rho_i, gamma, beta, g.d, s.y, y.y) lives in the field's device
// scalar block S, and a curvature pair with s.y <= 1e-12 y.y enters with
// rho = 0 (it then drops out of the recursion), so the host never waits for
// a dot product.  After each evaluation of E and its gradient at xt the
// caller reads back the block's tail (tail_at(m), kTail doubles: g.d, s.y,
// y.y, the 5 energy terms, the trial slope) and calls on_eval, which queues the vector operations
// that form the next trial point in xt; lbfgs_run runs them.
class Lbfgs {
 public:
  struct Bufs {
    double* x;   // accepted iterate
    double* xt;  // point to evaluate next
    double* g;   // gradient at x
    double* gt;  // gradient at xt (written by the evaluation)
    float* d;    // search direction
    float* hs;   // m stored steps s_i (n floats each)
    float* hy;   // m gradient changes y_i
    float* hinv; // diagonal preconditioner 1/D (written by the evaluation)
    double* S;   // nscalars(m) device scalars
    void* scratch;
  };
  enum Status { kRunning = -1, kConverged = 0, kFlat = 1, kMaxIter = 2, kStalled = 3 };
  static int nscalars(int m) { return 2 * m + 12; }
  static int tail_at(int m) { return 2 * m + 3; }
  static int energy_at(int m) { return 2 * m + 6; }  // 5 terms, then the trial slope g(xt) . d
  static constexpr int kTail = 9;                     // g.d, s.y, y.P.y, 5 terms, g(xt) . d

  // re-points the field's buffers (after a slot move the host state is kept)
  void bind(const Bufs& b, long long n, int m);
  // a new run from the point in xt: resets the scalars and the history.
  // e_noise > 0: the relative noise of E (an FP32 evaluation); a trial whose
  // E is within e_noise |E| of the current one and whose slope along the
  // direction has risen to at most (1 - 2 delta) |g.d| (approximate Wolfe,
  // Hager and Zhang 2005, delta = 0.1) is accepted when the Armijo test
  // cannot tell, so the run is not stopped by the noise; the evaluation must
  // then write g(xt) . d (energy_grad with the direction)
  void start(double gtol, double ftol, int max_iter, cudaStream_t s, double e_noise = 0.0);
  double e_noise() const { return e_noise_; }
  // the evaluation at xt is done: accept or backtrack, and queue the
  // operations of the next trial point into xt; true when the run has ended.
  // The caller runs ops() (lbfgs_run) after every call: when the run ends at
  // an accepted point they still keep that point in x.
  bool on_eval(const double* tail);
  long long size() const { return n_; }
  std::vector<LbOp>& ops() { return ops_; }
  int iterations() const { return iter_; }
  Status status() const { return status_; }
  const std::vector<double>& trace() const { return trace_; }  // 5 terms per accepted iterate
  const Bufs& bufs() const { return b_; }

 private:
  void direction();
  void step();
  void pass(float* x, const void* u, int u64, const void* v, int v64, double a0, int ja, double c0, double c1,
            int i1, double c2, int i2, double sc0, int js1, int js2, int out, const float* h = nullptr,
            int jh = -1);
  int alpha(int i) const { return i; }
  int rho(int i) const { return m_ + i; }
  int gamma() const { return 2 * m_; }
  int beta(int j) const { return 2 * m_ + 1 + (j & 1); }
  int gd() const { return 2 * m_ + 3; }

  Bufs b_{};
  long long n_ = 0;
  int m_ = 5;
  int nh_ = 0, head_ = 0, ls_ = 0, iter_ = 0, max_iter_ = 0;
  bool first_ = true;
  double gtol_ = 0, ftol_ = 0, t_ = 0, e_noise_ = 0;
  double E_[5] = {0, 0, 0, 0, 0};
  Status status_ = kRunning;
  std::vector<double> trace_;
  std::vector<LbOp> ops_;
};

}  // namespace mdft
