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
// may be null.  part / counter: reduction scratch (reduction_scratch_bytes,
// the counter zero, left zero).
void energy_grad(const EgConst& c, const double* xi, const void* vexc, bool vexc_f32, const double* vext,
                 const double* w, double* grad, long long n, int no, double* out, void* scratch, float* hinv,
                 cudaStream_t s);
size_t reduction_scratch_bytes();

// xi (double) -> float copy of n values
void to_float(float* y, const double* x, long long n, cudaStream_t s);

// L-BFGS (two-loop recursion with a diagonal initial inverse Hessian, the
// inverse local curvature; Armijo backtracking) of one field.  The host
// keeps only the line-search bookkeeping; every scalar of the recursion
// (alpha_i, rho_i, gamma, beta, g.d, s.y, y.y) lives in the field's device
// scalar block S, and a curvature pair with s.y <= 1e-12 y.y enters with
// rho = 0 (it then drops out of the recursion), so the host never waits for
// a dot product.  After each evaluation of E and its gradient at xt the
// caller reads back the block's tail (tail_at(m), 8 doubles: g.d, s.y, y.y,
// the 5 energy terms) and calls on_eval, which launches the next trial point
// into xt.
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
  static int nscalars(int m) { return 2 * m + 11; }
  static int tail_at(int m) { return 2 * m + 3; }
  static int energy_at(int m) { return 2 * m + 6; }

  // re-points the field's buffers (after a slot move the host state is kept)
  void bind(const Bufs& b, long long n, int m);
  // a new run from the point in xt: resets the scalars and the history
  void start(double gtol, double ftol, int max_iter, cudaStream_t s);
  // the evaluation at xt is done: accept or backtrack, and launch the next
  // trial point into xt; true when the run has ended
  bool on_eval(const double* tail, cudaStream_t s);
  int iterations() const { return iter_; }
  Status status() const { return status_; }
  const std::vector<double>& trace() const { return trace_; }  // 5 terms per accepted iterate
  const Bufs& bufs() const { return b_; }

 private:
  void direction(cudaStream_t s);
  void step(cudaStream_t s);
  template <typename TU, typename TV>
  void pass(float* x, const TU* u, const TV* v, double a0, int ja, double c1, int i1, double c2, int i2, double sc0,
            int js1, int js2, int out, cudaStream_t s, const float* h = nullptr, int jh = -1);
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
  double gtol_ = 0, ftol_ = 0, t_ = 0;
  double E_[5] = {0, 0, 0, 0, 0};
  Status status_ = kRunning;
  std::vector<double> trace_;
};

}  // namespace mdft
