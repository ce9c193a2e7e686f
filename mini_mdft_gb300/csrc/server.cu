// server.cu -- a job server for the excess-functional path.
//
// Jobs arrive from any host thread (mdft_server_submit) and are run by one
// worker thread that owns the GPU work:
//   * a job is one field on one grid with one solvent; each of its steps
//     evaluates the cproj excess energy and gradient at xi (get_delta_rho
//     fused into angl2proj, Convolution::execute, proj2angl, get_delta_f,
//     the stage sequence of Solver::energy_cproj_mrso,
//     src/mini-mdft.hpp:137-183) and then moves xi a fixed step down the
//     gradient; the job returns the energy of every step and its final xi;
//   * jobs with the same solvent and grid share a group: plans built once for
//     `max_batch` fields and a resident arena holding every field's xi, so
//     the group advances all its active jobs (compacted into the first k
//     slots) with one set of batched launches per step;
//   * each group step is replayed from a CUDA graph captured for its active
//     count k; the graphs of k = 1..16 are captured when the group is made
//     (a count whose capture fails, or a larger one, runs directly once and
//     is captured after that first direct step);
//   * a group is created only while the device memory of all groups stays
//     within the server's budget; groups without jobs are released, least
//     recently used first, when a new one does not fit;
//   * the server records every job's latency (submit to result) for p50/p99.
// No counterpart in the reference, which evaluates one field at a time.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "handles.hpp"
#include "solver.hpp"

using mdft::Error;
using mdft::throw_if;

namespace {

using Clock = std::chrono::steady_clock;

template <typename T>
__global__ void descent_kernel(T* __restrict__ xi, const T* __restrict__ df, const double* __restrict__ alpha,
                               long long per_field, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(i / per_field);
    xi[i] = xi[i] - (T)alpha[f] * df[i];
  }
}

// trace[j][step_j] = energy of slot j, step_j advanced (j < k)
__global__ void trace_kernel(const double* __restrict__ ff_cur, double* __restrict__ trace,
                             int* __restrict__ step_ctr, int k, int cap) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  const int s = step_ctr[j];
  if (s < cap) trace[(long long)j * cap + s] = ff_cur[j];
  step_ctr[j] = s + 1;
}

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(e == cudaErrorMemoryAllocation ? MDFT_ERR_NOMEM : MDFT_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
  }
}
void ckr(int rc, const char* what) {
  if (rc != MDFT_OK) throw Error(rc, std::string(what) + ": " + mdft_last_error());
}

struct Solvent {
  int mmax, mrso, np_luc, nq;
  double dq, rho0, prefactor;
  std::vector<int> luc_index;
  std::vector<double> luc;
  // molecular model for solute jobs: sites (q, sigma, epsilon, x, y, z), kT, vmax
  std::vector<double> sites;
  double kT = 0, vmax = 0;
};

// Page-locked host buffers for the job fields, kept for reuse: copies to and
// from pageable memory are staged by the driver at a fraction of the link's
// bandwidth, and page-locking on every job would cost more than the copy.
class PinnedPool {
 public:
  ~PinnedPool() {
    for (auto& kv : free_)
      for (void* p : kv.second) cudaFreeHost(p);
  }
  void* get(size_t bytes) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      auto it = free_.find(bytes);
      if (it != free_.end() && !it->second.empty()) {
        void* p = it->second.back();
        it->second.pop_back();
        return p;
      }
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      throw Error(MDFT_ERR_NOMEM, "page-locked host allocation failed");
    }
    return p;
  }
  void put(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    free_[bytes].push_back(p);
  }

 private:
  std::mutex mu_;
  std::map<size_t, std::vector<void*>> free_;
};

struct Job {
  long long id = 0;
  int solvent = 0;
  int n[3] = {0, 0, 0};
  double len[3] = {0, 0, 0};
  // initial field on submit, final field when done (page-locked, from the pool)
  void* xi = nullptr;
  size_t xi_bytes = 0;
  std::vector<double> ff;         // energy of every step
  int n_steps = 0;
  double step = 0;
  // solute jobs (kind 1): L-BFGS minimisation of the full functional
  int kind = 0;
  std::vector<double> solute;      // (q, sigma, epsilon, x, y, z) rows
  int max_iter = 0;
  double gtol = 0;
  std::vector<double> trace5;      // 5 terms per accepted iterate
  int iterations = 0, status = -1;
  int state = 0;  // 0 queued, 1 running, 2 done, -1 failed
  int code = 0;
  std::string error;
  Clock::time_point t_submit, t_done;
  int slot = -1, steps_done = 0;
};

using Key = std::tuple<int, int, int, int, int, double, double, double>;  // kind, solvent, grid

struct DevPtr {
  void* p = nullptr;
  ~DevPtr() {
    if (p) cudaFree(p);
  }
  void alloc(size_t bytes, const char* what) { ck(cudaMalloc(&p, bytes ? bytes : 1), what); }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

constexpr int kHistory = 5;  // L-BFGS pairs of a solute job

struct Group {
  Key key;
  int kind = 0;
  int B = 1, k = 0, prec = MDFT_F64, cap = 0;
  long long N = 0;
  int no = 0, np = 0;
  size_t elem = 8, bytes = 0;
  double rho0 = 0, prefactor = 0;
  mdft_grid_t grid = nullptr;
  mdft_opt_t opt = nullptr;
  mdft_conv_t conv = nullptr;
  DevPtr xi, vexc, df, p, w, ff_cur, trace, step_ctr, alpha, scratch;
  size_t scratch_per_slot = 0;
  // solute groups: per slot the minimiser's fields (xt contiguous: the batched
  // evaluation reads the k trial points as one array) and scalar blocks
  DevPtr xt, x, g, gt, vext, d, hs, hy, hinv, S, red;
  double* tails = nullptr;  // page-locked: Lbfgs::kTail doubles per slot read back each step
  std::vector<mdft::Lbfgs> lb;
  // every slot's L-BFGS operations of a step in one batch, one launch per
  // round (not the persistent cooperative launch: a group's launches share
  // the GPU with the other groups' streams)
  mdft::LbRunner lbr;
  int queued = 1;      // fixed-step groups: steps queued by the last launch
  mdft::EgConst eg{};
  Solvent model;
  cudaStream_t stream = nullptr;
  std::vector<std::shared_ptr<Job>> slots;  // active jobs, slot i = field i
  std::map<int, cudaGraphExec_t> graphs;    // per active count; null: run directly
  std::map<int, int> seen;                  // steps run directly at each active count
  bool inflight = false;                    // a step is queued on the stream
  Clock::time_point last_used;
  ~Group() {
    if (tails) cudaFreeHost(tails);
    for (auto& g : graphs)
      if (g.second) cudaGraphExecDestroy(g.second);
    if (stream) cudaStreamDestroy(stream);
    if (conv) mdft_conv_destroy(conv);
    if (opt) mdft_opt_destroy(opt);
    if (grid) mdft_grid_destroy(grid);
  }
};

}  // namespace

struct mdft_server_s {
  int device = 0, prec = MDFT_F64, max_batch = 1, trace_cap = 4096;
  size_t budget = 0, in_use = 0;  // in_use: worker only
  std::atomic<size_t> peak{0};
  std::atomic<int> n_groups{0};
  std::atomic<long long> graph_steps{0}, direct_steps{0};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Job>> incoming;
  std::map<long long, std::shared_ptr<Job>> jobs;
  std::vector<Solvent> solvents;
  PinnedPool pinned;
  long long next_id = 1;
  bool stop = false;
  std::thread worker;
  // statistics (under mu)
  std::vector<double> latencies;
  bool any_submit = false;
  Clock::time_point t_first_submit, t_last_done;
  // worker-only state
  std::vector<std::shared_ptr<Job>> pending;
  std::map<Key, std::unique_ptr<Group>> groups;

  void run();
  void admit();
  Group* group_for(const Job& j);
  void step(Group& g);
  void precapture(Group& g);
  void enqueue_step(Group& g, int k);
  void bind_slot(Group& g, int slot);
  void complete_step(Group& g);
  void finish(Group& g, int slot);
  void fail_group(Group& g, const std::string& msg, int code);
  void fail_job(const std::shared_ptr<Job>& j, const std::string& msg, int code);
};

namespace {

size_t field_bytes(const Group& g) { return (size_t)g.N * g.no * g.elem; }

}  // namespace

void mdft_server_s::fail_job(const std::shared_ptr<Job>& j, const std::string& msg, int code) {
  std::lock_guard<std::mutex> lk(mu);
  j->state = -1;
  j->code = code ? code : MDFT_ERR_INVALID;
  j->error = msg;
  j->t_done = Clock::now();
  cv_done.notify_all();
}

void mdft_server_s::fail_group(Group& g, const std::string& msg, int code) {
  for (auto& j : g.slots) fail_job(j, msg, code);
  g.slots.clear();
  g.k = 0;
}

Group* mdft_server_s::group_for(const Job& j) {
  const Key key{j.kind, j.solvent, j.n[0], j.n[1], j.n[2], j.len[0], j.len[1], j.len[2]};
  auto it = groups.find(key);
  if (it != groups.end()) return it->second.get();
  Solvent sv;
  {
    std::lock_guard<std::mutex> lk(mu);  // add_solvent may grow the list meanwhile
    sv = solvents[j.solvent];
  }
  // footprint: plans (measured) + arena (computed); admit only within budget
  auto g = std::make_unique<Group>();
  g->key = key;
  g->kind = j.kind;
  g->B = max_batch;
  g->prec = prec;
  g->cap = trace_cap;
  g->elem = prec == MDFT_F32 ? 4 : 8;
  g->rho0 = sv.rho0;
  g->prefactor = sv.prefactor;
  ckr(mdft_grid_create(&g->grid, j.n[0], j.n[1], j.n[2], j.len[0], j.len[1], j.len[2], sv.mmax, sv.mrso),
      "job grid");
  int info[11];
  ckr(mdft_grid_info(g->grid, info), "grid info");
  g->N = (long long)j.n[0] * j.n[1] * j.n[2];
  g->no = info[8];
  g->np = info[9];
  const size_t fb = field_bytes(*g);
  const size_t nbp = mdft::delta_f_partials((size_t)g->N, g->no);
  g->scratch_per_slot = (sizeof(double2) * nbp + 256 + 255) / 256 * 256;
  const size_t f64b = (size_t)g->N * g->no * 8;  // one FP64 field
  const size_t arena =
      g->kind == 0 ? 3 * fb * g->B + (size_t)g->np * g->N * 2 * g->elem * g->B + g->scratch_per_slot * g->B +
                         (size_t)g->B * (g->cap + 3) * 8 + 8 * g->no
                   : (5 * f64b + f64b / 2 * (2 + 2 * kHistory) + fb * (g->elem == 4 ? 2 : 1) +
                      (size_t)g->np * g->N * 2 * g->elem) *
                             g->B +
                         mdft::reduction_scratch_bytes() * g->B + 8 * g->no;
  // a rough bound on the plans before building them: the R(q) table and
  // pair data dominate (about 1 KB per grid point at mmax <= 6)
  const size_t plan_guess = (size_t)g->N * 1024;
  if (in_use + arena + plan_guess > budget) {
    // release idle groups, least recently used first
    std::vector<std::pair<Clock::time_point, Key>> idle;
    for (auto& kv : groups)
      if (kv.second->k == 0) idle.push_back({kv.second->last_used, kv.first});
    std::sort(idle.begin(), idle.end());
    for (auto& e : idle) {
      if (in_use + arena + plan_guess <= budget) break;
      in_use -= groups[e.second]->bytes;
      groups.erase(e.second);
      n_groups.store((int)groups.size());
    }
    if (in_use + arena + plan_guess > budget) {
      bool busy = false;
      for (auto& kv : groups) busy = busy || kv.second->k > 0;
      if (!busy)
        throw Error(MDFT_ERR_NOMEM, "job needs about " + std::to_string((arena + plan_guess) >> 20) +
                                        " MiB of device memory, over the server's budget of " +
                                        std::to_string(budget >> 20) + " MiB");
      return nullptr;  // wait for running groups to finish
    }
  }
  size_t free0 = 0, free1 = 0, total = 0;
  ck(cudaMemGetInfo(&free0, &total), "cudaMemGetInfo");
  ckr(mdft_opt_create_batched(&g->opt, g->grid, prec, g->B), "job plan (angular)");
  ckr(mdft_conv_create_batched(&g->conv, g->grid, sv.luc_index.data(), sv.luc.data(), sv.np_luc, sv.nq, sv.dq,
                               prec, g->B),
      "job plan (convolution)");
  g->vexc.alloc(fb * g->B, "server arena");
  g->p.alloc((size_t)g->np * g->N * 2 * g->elem * g->B, "server arena");
  if (g->kind == 0) {
    g->xi.alloc(fb * g->B, "server arena");
    g->df.alloc(fb * g->B, "server arena");
    g->scratch.alloc(g->scratch_per_slot * g->B, "server arena");
    g->trace.alloc((size_t)g->B * g->cap * 8, "server arena");
    g->ff_cur.alloc((size_t)g->B * 8, "server arena");
    g->alpha.alloc((size_t)g->B * 8, "server arena");
    g->step_ctr.alloc((size_t)g->B * 4, "server arena");
  } else {
    if (g->elem == 4) g->xi.alloc(fb * g->B, "server arena");  // FP32 copy of the trial points
    for (DevPtr* f : {&g->xt, &g->x, &g->g, &g->gt, &g->vext}) f->alloc(f64b * g->B, "server arena");
    g->d.alloc(f64b / 2 * g->B, "server arena");
    g->hinv.alloc(f64b / 2 * g->B, "server arena");
    g->hs.alloc(f64b / 2 * kHistory * g->B, "server arena");
    g->hy.alloc(f64b / 2 * kHistory * g->B, "server arena");
    g->S.alloc(sizeof(double) * mdft::Lbfgs::nscalars(kHistory) * g->B, "server arena");
    g->red.alloc(mdft::reduction_scratch_bytes() * g->B, "server arena");  // one per slot
    ck(cudaMemset(g->red.p, 0, mdft::reduction_scratch_bytes() * g->B), "scratch reset");
    ck(cudaHostAlloc((void**)&g->tails, sizeof(double) * mdft::Lbfgs::kTail * g->B, cudaHostAllocDefault),
       "page-locked tails");
    g->lbr.rounds = true;
    g->lb.resize(g->B);
    g->model = sv;
    g->eg = mdft::EgConst{sv.kT, sv.rho0, (j.len[0] / j.n[0]) * (j.len[1] / j.n[1]) * (j.len[2] / j.n[2]),
                          sv.prefactor};
  }
  g->w.alloc((size_t)g->no * 8, "server arena");
  std::vector<double> th(info[5]), wth(info[5]), w(g->no);
  ckr(mdft_grid_angular(g->grid, th.data(), wth.data(), w.data()), "angular weights");
  ck(cudaMemcpy(g->w.p, w.data(), 8 * g->no, cudaMemcpyHostToDevice), "weights upload");
  ck(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  ck(cudaMemGetInfo(&free1, &total), "cudaMemGetInfo");
  g->bytes = free0 > free1 ? free0 - free1 : arena;
  in_use += g->bytes;
  if (in_use > peak.load()) peak.store(in_use);
  precapture(*g);
  Group* raw = g.get();
  groups.emplace(key, std::move(g));
  n_groups.store((int)groups.size());
  return raw;
}

void mdft_server_s::admit() {
  std::vector<std::shared_ptr<Job>> keep;
  for (auto& j : pending) {
    Group* g = nullptr;
    try {
      g = group_for(*j);
    } catch (const Error& e) {
      fail_job(j, e.what(), e.code);
      continue;
    }
    if (!g || g->k >= g->B || g->inflight) {
      keep.push_back(j);
      continue;
    }
    const int slot = g->k;
    try {
      if (g->kind == 0) {
        const size_t fb = field_bytes(*g);
        ck(cudaMemcpyAsync(g->xi.as<unsigned char>() + fb * slot, j->xi, fb, cudaMemcpyHostToDevice, g->stream),
           "job field upload");
        ck(cudaMemcpyAsync(g->alpha.as<double>() + slot, &j->step, 8, cudaMemcpyHostToDevice, g->stream),
           "job step upload");
        ck(cudaMemsetAsync(g->step_ctr.as<int>() + slot, 0, 4, g->stream), "job counter reset");
      } else {
        // start point, the job's external potential, a fresh minimiser
        const long long n = g->N * g->no;
        ck(cudaMemcpyAsync(g->xt.as<double>() + (size_t)n * slot, j->xi, sizeof(double) * n, cudaMemcpyHostToDevice,
                           g->stream),
           "job field upload");
        mdft::vext_compute(g->grid->g, g->model.sites.data(), (int)g->model.sites.size() / 6,
                           j->solute.data(), (int)j->solute.size() / 6, g->model.vmax,
                           g->vext.as<double>() + (size_t)n * slot, g->stream);
        bind_slot(*g, slot);
        // the FP32 form's energies are noisy at ~1e-7: accept by the slope too
        g->lb[slot].start(j->gtol, 0.0, j->max_iter, g->stream, g->elem == 4 ? 1e-6 : 0.0);
      }
      ck(cudaStreamSynchronize(g->stream), "job admission");
    } catch (const Error& e) {
      fail_job(j, e.what(), e.code);
      continue;
    }
    j->slot = slot;
    j->steps_done = 0;
    {
      std::lock_guard<std::mutex> lk(mu);
      j->state = 1;
    }
    g->slots.push_back(j);
    g->k += 1;
    g->last_used = Clock::now();
  }
  pending.swap(keep);
}

void mdft_server_s::bind_slot(Group& g, int slot) {
  const size_t n = (size_t)g.N * g.no;
  const int ns = mdft::Lbfgs::nscalars(kHistory);
  g.lb[slot].bind(mdft::Lbfgs::Bufs{g.x.as<double>() + n * slot, g.xt.as<double>() + n * slot,
                                    g.g.as<double>() + n * slot, g.gt.as<double>() + n * slot,
                                    g.d.as<float>() + n * slot, g.hs.as<float>() + n * kHistory * slot,
                                    g.hy.as<float>() + n * kHistory * slot, g.hinv.as<float>() + n * slot,
                                    g.S.as<double>() + (size_t)ns * slot, g.red.p},
                  (long long)n, kHistory);
}

// Solute groups: the energy and gradient of every active job at its trial
// point (one batched cproj evaluation), and each job's scalar tail read back;
// the minimisers then choose the next trial points on the host.
void enqueue_solve_step(Group& g, int k) {
  cudaStream_t s = g.stream;
  const size_t n = (size_t)g.N * g.no;
  const void* xin = g.xt.p;
  if (g.elem == 4) {
    mdft::to_float(g.xi.as<float>(), g.xt.as<double>(), (long long)n * k, s);
    xin = g.xi.p;
  }
  mdft::detail::angl2proj_fields(g.opt, xin, true, g.rho0, g.p.p, k, s);
  mdft::detail::execute_fields(g.conv, g.p.p, k, s);
  mdft::detail::proj2angl_fields(g.opt, g.p.p, g.vexc.p, k, s);
  // every slot's energy, gradient and preconditioner in one launch, then the
  // slots' scalar tails (kTail doubles each, one scalar block apart) in one
  // copy; the FP32 form also sums each slot's slope along its direction
  const int ns = mdft::Lbfgs::nscalars(kHistory);
  mdft::energy_grad(g.eg, g.xt.as<double>(), g.vexc.p, g.elem == 4, g.vext.as<double>(), g.w.as<double>(),
                    g.gt.as<double>(), (long long)n, g.no, g.S.as<double>() + mdft::Lbfgs::energy_at(kHistory),
                    g.red.p, g.hinv.as<float>(), s, k, ns, g.elem == 4 ? g.d.as<float>() : nullptr);
  constexpr size_t tb = sizeof(double) * mdft::Lbfgs::kTail;
  ck(cudaMemcpy2DAsync(g.tails, tb, g.S.as<double>() + mdft::Lbfgs::tail_at(kHistory), sizeof(double) * ns, tb, k,
                       cudaMemcpyDeviceToHost, s),
     "minimiser tail read-back");
}

void mdft_server_s::enqueue_step(Group& g, int k) {
  if (g.kind == 1) {
    enqueue_solve_step(g, k);
    return;
  }
  cudaStream_t s = g.stream;
  mdft::detail::angl2proj_fields(g.opt, g.xi.p, true, g.rho0, g.p.p, k, s);
  mdft::detail::execute_fields(g.conv, g.p.p, k, s);
  mdft::detail::proj2angl_fields(g.opt, g.p.p, g.vexc.p, k, s);
  // the energy reduction's completion counters start at zero
  ck(cudaMemsetAsync(g.scratch.p, 0, g.scratch_per_slot * k, s), "energy scratch reset");
  const size_t fb = field_bytes(g);
  for (int j = 0; j < k; ++j) {
    unsigned char* sc = g.scratch.as<unsigned char>() + g.scratch_per_slot * j;
    if (g.elem == 8)
      mdft::launch_delta_f<double>(
          reinterpret_cast<const double*>(g.xi.as<unsigned char>() + fb * j),
          reinterpret_cast<const double*>(g.vexc.as<unsigned char>() + fb * j), g.w.as<double>(),
          reinterpret_cast<double*>(g.df.as<unsigned char>() + fb * j), g.ff_cur.as<double>() + j, (size_t)g.N,
          g.no, g.rho0, g.prefactor, sc, s, g.prec == MDFT_F64);
    else
      mdft::launch_delta_f<float>(
          reinterpret_cast<const float*>(g.xi.as<unsigned char>() + fb * j),
          reinterpret_cast<const float*>(g.vexc.as<unsigned char>() + fb * j), g.w.as<double>(),
          reinterpret_cast<float*>(g.df.as<unsigned char>() + fb * j), g.ff_cur.as<double>() + j, (size_t)g.N,
          g.no, g.rho0, g.prefactor, sc, s, false);
  }
  trace_kernel<<<(k + 127) / 128, 128, 0, s>>>(g.ff_cur.as<double>(), g.trace.as<double>(), g.step_ctr.as<int>(), k,
                                                g.cap);
  mdft::launch_check("server trace kernel launch");
  const long long per_field = g.N * g.no, n = per_field * k;
  const unsigned nb = (unsigned)std::min<long long>((n + 255) / 256, 152LL * 16);
  if (g.elem == 8)
    descent_kernel<double><<<nb, 256, 0, s>>>(g.xi.as<double>(), g.df.as<double>(), g.alpha.as<double>(),
                                              per_field, n);
  else
    descent_kernel<float><<<nb, 256, 0, s>>>(g.xi.as<float>(), g.df.as<float>(), g.alpha.as<double>(), per_field,
                                             n);
  mdft::launch_check("server descent kernel launch");
}

// Captures the step graphs of the active counts 1..min(B, kPrecapture) of a
// new group, so that no capture or instantiation lands in a running job's
// step; a count whose capture fails, or a larger one, runs directly at its
// first step and is captured at its second (step()).
constexpr int kPrecapture = 16;
void mdft_server_s::precapture(Group& g) {
  for (int k = 1; k <= std::min(g.B, kPrecapture); ++k) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool ok = cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      try {
        enqueue_step(g, k);
      } catch (const Error&) {
        ok = false;
      }
      ok = (cudaStreamEndCapture(g.stream, &graph) == cudaSuccess) && ok && graph;
      ok = ok && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
    }
    cudaGetLastError();
    if (ok) g.graphs[k] = exec;
  }
}

void mdft_server_s::step(Group& g) {
  const int k = g.k;
  auto it = g.graphs.find(k);
  if (it != g.graphs.end() && it->second) {
    ck(cudaGraphLaunch(it->second, g.stream), "cudaGraphLaunch");
    graph_steps += 1;
    return;
  }
  if (it == g.graphs.end() && g.seen[k] >= 1) {
    // capture this active count once; on any failure run it directly from now on
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool ok = cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      try {
        enqueue_step(g, k);
      } catch (const Error&) {
        ok = false;
      }
      ok = (cudaStreamEndCapture(g.stream, &graph) == cudaSuccess) && ok && graph;
      ok = ok && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      if (graph) cudaGraphDestroy(graph);
    }
    cudaGetLastError();
    g.graphs[k] = ok ? exec : nullptr;
    if (ok) {
      ck(cudaGraphLaunch(exec, g.stream), "cudaGraphLaunch");
      graph_steps += 1;
      return;
    }
  }
  g.seen[k] += 1;
  enqueue_step(g, k);
  direct_steps += 1;
}

void mdft_server_s::finish(Group& g, int slot) {
  std::shared_ptr<Job> j = g.slots[slot];
  if (g.kind == 1) {
    const size_t n = (size_t)g.N * g.no;
    ck(cudaMemcpyAsync(j->xi, g.x.as<double>() + n * slot, sizeof(double) * n, cudaMemcpyDeviceToHost, g.stream),
       "job field download");
    std::vector<double> tr = g.lb[slot].trace();
    const int iters = g.lb[slot].iterations(), status = (int)g.lb[slot].status();
    const int last = g.k - 1;
    if (slot != last) {  // the last active job moves into the freed slot
      const int ns = mdft::Lbfgs::nscalars(kHistory);
      auto mv = [&](DevPtr& f, size_t per) {
        ck(cudaMemcpyAsync(f.as<unsigned char>() + per * slot, f.as<unsigned char>() + per * last, per,
                           cudaMemcpyDeviceToDevice, g.stream),
           "slot move");
      };
      for (DevPtr* f : {&g.xt, &g.x, &g.g, &g.gt, &g.vext}) mv(*f, 8 * n);
      mv(g.d, 4 * n);
      mv(g.hinv, 4 * n);
      mv(g.hs, 4 * n * kHistory);
      mv(g.hy, 4 * n * kHistory);
      mv(g.S, 8 * (size_t)ns);
      g.lb[slot] = g.lb[last];
      bind_slot(g, slot);
      g.slots[slot] = g.slots[last];
      g.slots[slot]->slot = slot;
    }
    ck(cudaStreamSynchronize(g.stream), "job completion");
    g.slots.pop_back();
    g.k -= 1;
    g.last_used = Clock::now();
    std::lock_guard<std::mutex> lk(mu);
    j->trace5.swap(tr);
    j->iterations = iters;
    j->status = status;
    j->state = 2;
    j->t_done = Clock::now();
    latencies.push_back(std::chrono::duration<double>(j->t_done - j->t_submit).count());
    t_last_done = j->t_done;
    cv_done.notify_all();
    return;
  }
  const size_t fb = field_bytes(g);
  std::vector<double> ff(j->n_steps);
  // the final field goes back into the job's page-locked buffer
  ck(cudaMemcpyAsync(j->xi, g.xi.as<unsigned char>() + fb * slot, fb, cudaMemcpyDeviceToHost, g.stream),
     "job field download");
  ck(cudaMemcpyAsync(ff.data(), g.trace.as<double>() + (size_t)slot * g.cap, 8 * (size_t)j->n_steps,
                     cudaMemcpyDeviceToHost, g.stream),
     "job energies download");
  // keep the active slots compact: the last one moves into the freed slot
  const int last = g.k - 1;
  if (slot != last) {
    ck(cudaMemcpyAsync(g.xi.as<unsigned char>() + fb * slot, g.xi.as<unsigned char>() + fb * last, fb,
                       cudaMemcpyDeviceToDevice, g.stream),
       "slot move");
    ck(cudaMemcpyAsync(g.trace.as<double>() + (size_t)slot * g.cap, g.trace.as<double>() + (size_t)last * g.cap,
                       8 * (size_t)g.cap, cudaMemcpyDeviceToDevice, g.stream),
       "slot move");
    ck(cudaMemcpyAsync(g.alpha.as<double>() + slot, g.alpha.as<double>() + last, 8, cudaMemcpyDeviceToDevice,
                       g.stream),
       "slot move");
    ck(cudaMemcpyAsync(g.step_ctr.as<int>() + slot, g.step_ctr.as<int>() + last, 4, cudaMemcpyDeviceToDevice,
                       g.stream),
       "slot move");
    g.slots[slot] = g.slots[last];
    g.slots[slot]->slot = slot;
  }
  ck(cudaStreamSynchronize(g.stream), "job completion");
  g.slots.pop_back();
  g.k -= 1;
  g.last_used = Clock::now();
  std::lock_guard<std::mutex> lk(mu);
  j->ff.swap(ff);
  j->state = 2;
  j->t_done = Clock::now();
  latencies.push_back(std::chrono::duration<double>(j->t_done - j->t_submit).count());
  t_last_done = j->t_done;
  cv_done.notify_all();
}

void mdft_server_s::run() {
  cudaSetDevice(device);
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu);
      auto busy = [&] {
        for (auto& kv : groups)
          if (kv.second->k > 0 || kv.second->inflight) return true;
        return false;
      };
      cv_work.wait(lk, [&] { return stop || !incoming.empty() || busy() || !pending.empty(); });
      if (stop) return;
      while (!incoming.empty()) {
        pending.push_back(incoming.front());
        incoming.pop_front();
      }
    }
    // Each group advances on its own: a group whose step has finished takes
    // its results, refills its free slots from the queue, and launches its
    // next step at once, without waiting for the other groups' steps (small
    // grids step several times per step of a large one, and the groups'
    // work overlaps on the device).
    bool progress = false, live = false;
    for (auto& kv : groups) {
      Group* g = kv.second.get();
      if (!g->inflight) continue;
      const cudaError_t q = cudaStreamQuery(g->stream);
      if (q == cudaErrorNotReady) {
        live = true;
        continue;
      }
      g->inflight = false;
      progress = true;
      try {
        ck(q, "server step");
        mdft::check_device_waits();  // a persistent launch whose barrier ran out fails the group
        complete_step(*g);
      } catch (const Error& e) {
        fail_group(*g, e.what(), e.code);
      }
    }
    admit();  // every group not in flight takes queued jobs into its free slots
    for (auto& kv : groups) {
      Group* g = kv.second.get();
      if (g->inflight || g->k == 0) continue;
      live = true;
      try {
        // fixed-step jobs: queue as many steps as the active job closest to
        // its end still needs (one host round trip for all of them)
        int r = 1;
        if (g->kind == 0) {
          r = 1 << 30;
          for (auto& j : g->slots) r = std::min(r, j->n_steps - j->steps_done);
          r = std::max(1, r);
        }
        g->queued = r;
        for (int q = 0; q < r; ++q) step(*g);
        g->inflight = true;
        progress = true;
      } catch (const Error& e) {
        fail_group(*g, e.what(), e.code);
      }
    }
    if (!live) {
      // queued jobs that cannot be placed yet and nothing running: wait for news
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait_for(lk, std::chrono::milliseconds(2), [&] { return stop || !incoming.empty(); });
    } else if (!progress) {
      std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
  }
}

// The group's step has finished: every job records it, solute jobs' minimisers
// queue their next trial points, finished jobs leave.
void mdft_server_s::complete_step(Group& g) {
  for (auto& j : g.slots) j->steps_done += g.kind == 1 ? 1 : g.queued;
  if (g.kind == 1) {
    // every slot's minimiser decides on the host and queues its vector
    // operations; one persistent launch runs them all; then the ended jobs
    // leave, highest slot first, so that a finished job's slot is refilled by
    // a job that has already queued its own next point
    std::vector<int> ended;
    std::vector<mdft::Lbfgs*> run;
    for (int s = g.k - 1; s >= 0; --s) {
      if (g.lb[s].on_eval(g.tails + mdft::Lbfgs::kTail * s)) ended.push_back(s);
      run.push_back(&g.lb[s]);
    }
    mdft::lbfgs_run(run.data(), (int)run.size(), g.lbr, g.stream);
    for (int s : ended) finish(g, s);
  } else {
    for (int s = g.k - 1; s >= 0; --s)
      if (g.slots[s]->steps_done >= g.slots[s]->n_steps) finish(g, s);
  }
}

// ---- C ABI --------------------------------------------------------------------
namespace {
template <typename F>
int sguard(F&& f) {
  try {
    f();
    return MDFT_OK;
  } catch (const Error& e) {
    return mdft::record_error(e.code, e.what());
  } catch (const std::bad_alloc&) {
    return mdft::record_error(MDFT_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& e) {
    return mdft::record_error(MDFT_ERR_INVALID, e.what());
  }
}
}  // namespace

int mdft_server_create(mdft_server_t* out, int precision, int max_batch, size_t hbm_budget_bytes) {
  return sguard([&] {
    throw_if(!out, "NULL argument");
    *out = nullptr;
    throw_if(precision != MDFT_F64 && precision != MDFT_F32 && precision != MDFT_F64_DF,
             "precision must be MDFT_F64, MDFT_F32 or MDFT_F64_DF");
    throw_if(max_batch < 1 || max_batch > 1024, "max_batch must be 1..1024");
    auto s = std::make_unique<mdft_server_s>();
    s->device = mdft::detail::current_device();
    s->prec = precision;
    s->max_batch = max_batch;
    size_t free_b = 0, total = 0;
    ck(cudaMemGetInfo(&free_b, &total), "cudaMemGetInfo");
    s->budget = hbm_budget_bytes ? hbm_budget_bytes : free_b / 10 * 8;
    mdft_server_s* raw = s.get();
    s->worker = std::thread([raw] { raw->run(); });
    *out = s.release();
  });
}

int mdft_server_destroy(mdft_server_t s) {
  if (!s) return MDFT_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    for (auto& kv : s->jobs)
      if (kv.second->state == 0 || kv.second->state == 1) {
        kv.second->state = -1;
        kv.second->code = MDFT_ERR_INVALID;
        kv.second->error = "server destroyed";
      }
    s->cv_done.notify_all();
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->device);
  for (auto& kv : s->jobs) {  // results never collected: their buffers go back to the pool
    s->pinned.put(kv.second->xi, kv.second->xi_bytes);
    kv.second->xi = nullptr;
  }
  delete s;
  return MDFT_OK;
}

int mdft_server_add_solvent(mdft_server_t s, int mmax, int mrso, const int* luc_index, const double* luc,
                            int np_luc, int nq, double dq, double rho0, double prefactor, int* solvent_id) {
  return sguard([&] {
    throw_if(!s || !luc_index || !luc || !solvent_id, "NULL argument");
    throw_if(mmax < 1 || mmax > 6 || mrso < 1, "solvent needs 1 <= mmax <= 6 and mrso >= 1");
    throw_if(np_luc <= 0 || nq <= 1 || !(dq > 0), "invalid c(q) table extents");
    Solvent sv;
    sv.mmax = mmax;
    sv.mrso = mrso;
    sv.np_luc = np_luc;
    sv.nq = nq;
    sv.dq = dq;
    sv.rho0 = rho0;
    sv.prefactor = prefactor;
    sv.luc_index.assign(luc_index, luc_index + 5 * (size_t)np_luc);
    sv.luc.assign(luc, luc + 2 * (size_t)np_luc * nq);
    std::lock_guard<std::mutex> lk(s->mu);
    s->solvents.push_back(std::move(sv));
    *solvent_id = (int)s->solvents.size() - 1;
  });
}

int mdft_server_submit(mdft_server_t s, int solvent_id, int nx, int ny, int nz, double lx, double ly, double lz,
                       const void* xi0, int n_steps, double step, long long* job_id) {
  return sguard([&] {
    throw_if(!s || !xi0 || !job_id, "NULL argument");
    throw_if(nx < 1 || ny < 1 || nz < 1 || !(lx > 0) || !(ly > 0) || !(lz > 0), "invalid grid");
    throw_if(n_steps < 1 || n_steps > s->trace_cap, "n_steps must be 1.." + std::to_string(s->trace_cap));
    auto j = std::make_shared<Job>();
    int no = 0;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      throw_if(solvent_id < 0 || solvent_id >= (int)s->solvents.size(), "unknown solvent");
      const Solvent& sv = s->solvents[solvent_id];
      const int nt = sv.mmax + 1, nphi = 2 * sv.mmax + 1, npsi = 2 * (sv.mmax / sv.mrso) + 1;
      no = nt * nphi * npsi;
    }
    const size_t elem = s->prec == MDFT_F32 ? 4 : 8;
    const size_t bytes = (size_t)nx * ny * nz * no * elem;
    j->solvent = solvent_id;
    j->n[0] = nx;
    j->n[1] = ny;
    j->n[2] = nz;
    j->len[0] = lx;
    j->len[1] = ly;
    j->len[2] = lz;
    j->xi = s->pinned.get(bytes);
    j->xi_bytes = bytes;
    std::memcpy(j->xi, xi0, bytes);
    j->n_steps = n_steps;
    j->step = step;
    j->t_submit = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      j->id = s->next_id++;
      if (!s->any_submit) {
        s->any_submit = true;
        s->t_first_submit = j->t_submit;
      }
      s->jobs[j->id] = j;
      s->incoming.push_back(j);
      *job_id = j->id;
    }
    s->cv_work.notify_all();
  });
}

int mdft_server_wait(mdft_server_t s, long long job_id, void* xi_out, double* ff_out, double* latency_s) {
  return sguard([&] {
    throw_if(!s, "NULL argument");
    std::shared_ptr<Job> j;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    throw_if(it == s->jobs.end(), "unknown job (or its result was already taken)");
    j = it->second;
    s->cv_done.wait(lk, [&] { return j->state == 2 || j->state == -1; });
    s->jobs.erase(it);
    lk.unlock();
    struct Release {  // the buffer returns to the pool however this ends
      mdft_server_s* s;
      std::shared_ptr<Job> j;
      ~Release() {
        s->pinned.put(j->xi, j->xi_bytes);
        j->xi = nullptr;
      }
    } rel{s, j};
    if (j->state == -1) throw Error(j->code, j->error);
    throw_if(j->kind != 0, "a solute job: collect it with mdft_server_wait_solute");
    if (xi_out) std::memcpy(xi_out, j->xi, j->xi_bytes);
    if (ff_out) std::memcpy(ff_out, j->ff.data(), sizeof(double) * j->ff.size());
    if (latency_s) *latency_s = std::chrono::duration<double>(j->t_done - j->t_submit).count();
  });
}

int mdft_server_set_solvent_model(mdft_server_t s, int solvent_id, const double* sites, int n_sites, double kT,
                                  double vmax) {
  return sguard([&] {
    throw_if(!s || !sites, "NULL argument");
    throw_if(n_sites < 1, "a solvent model needs at least one site");
    throw_if(!(kT > 0) || !(vmax > 0), "kT and vmax must be positive");
    std::lock_guard<std::mutex> lk(s->mu);
    throw_if(solvent_id < 0 || solvent_id >= (int)s->solvents.size(), "unknown solvent");
    Solvent& sv = s->solvents[solvent_id];
    sv.sites.assign(sites, sites + 6 * (size_t)n_sites);
    sv.kT = kT;
    sv.vmax = vmax;
  });
}

int mdft_server_submit_solute(mdft_server_t s, int solvent_id, int nx, int ny, int nz, double lx, double ly,
                              double lz, const double* solute_sites, int n_sites, const double* xi0, int max_iter,
                              double gtol, long long* job_id) {
  return sguard([&] {
    throw_if(!s || !job_id || (n_sites > 0 && !solute_sites), "NULL argument");
    throw_if(nx < 1 || ny < 1 || nz < 1 || !(lx > 0) || !(ly > 0) || !(lz > 0), "invalid grid");
    throw_if(n_sites < 0, "n_sites must be >= 0");
    throw_if(max_iter < 0 || max_iter > 100000, "max_iter must be 0..100000");
    throw_if(!(gtol >= 0), "gtol must be >= 0");
    auto j = std::make_shared<Job>();
    int no = 0;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      throw_if(solvent_id < 0 || solvent_id >= (int)s->solvents.size(), "unknown solvent");
      const Solvent& sv = s->solvents[solvent_id];
      throw_if(sv.sites.empty(), "the solvent has no molecular model (mdft_server_set_solvent_model)");
      const int nt = sv.mmax + 1, nphi = 2 * sv.mmax + 1, npsi = 2 * (sv.mmax / sv.mrso) + 1;
      no = nt * nphi * npsi;
    }
    const size_t n = (size_t)nx * ny * nz * no, bytes = n * sizeof(double);
    j->kind = 1;
    j->solvent = solvent_id;
    j->n[0] = nx;
    j->n[1] = ny;
    j->n[2] = nz;
    j->len[0] = lx;
    j->len[1] = ly;
    j->len[2] = lz;
    j->solute.assign(solute_sites, solute_sites + 6 * (size_t)n_sites);
    j->max_iter = max_iter;
    j->gtol = gtol;
    j->xi = s->pinned.get(bytes);
    j->xi_bytes = bytes;
    if (xi0) {
      std::memcpy(j->xi, xi0, bytes);
    } else {
      double* x = static_cast<double*>(j->xi);
      std::fill(x, x + n, 1.0);  // the bulk density
    }
    j->t_submit = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      j->id = s->next_id++;
      if (!s->any_submit) {
        s->any_submit = true;
        s->t_first_submit = j->t_submit;
      }
      s->jobs[j->id] = j;
      s->incoming.push_back(j);
      *job_id = j->id;
    }
    s->cv_work.notify_all();
  });
}

int mdft_server_wait_solute(mdft_server_t s, long long job_id, double* xi_out, double* trace_out, int* iterations,
                            int* status, double* latency_s) {
  return sguard([&] {
    throw_if(!s, "NULL argument");
    std::shared_ptr<Job> j;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job_id);
    throw_if(it == s->jobs.end(), "unknown job (or its result was already taken)");
    j = it->second;
    s->cv_done.wait(lk, [&] { return j->state == 2 || j->state == -1; });
    s->jobs.erase(it);
    lk.unlock();
    struct Release {
      mdft_server_s* s;
      std::shared_ptr<Job> j;
      ~Release() {
        s->pinned.put(j->xi, j->xi_bytes);
        j->xi = nullptr;
      }
    } rel{s, j};
    if (j->state == -1) throw Error(j->code, j->error);
    throw_if(j->kind != 1, "not a solute job: collect it with mdft_server_wait");
    if (xi_out) std::memcpy(xi_out, j->xi, j->xi_bytes);
    if (trace_out) std::memcpy(trace_out, j->trace5.data(), sizeof(double) * j->trace5.size());
    if (iterations) *iterations = j->iterations;
    if (status) *status = j->status;
    if (latency_s) *latency_s = std::chrono::duration<double>(j->t_done - j->t_submit).count();
  });
}

int mdft_server_stats(mdft_server_t s, double* out) {
  return sguard([&] {
    throw_if(!s || !out, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
      if (l.empty()) return 0.0;
      const size_t i = (size_t)std::min<double>((double)l.size() - 1, std::ceil(q * l.size()) - 1);
      return l[i];
    };
    const double span =
        l.empty() ? 0.0 : std::chrono::duration<double>(s->t_last_done - s->t_first_submit).count();
    out[0] = (double)l.size();
    out[1] = span > 0 ? l.size() / span : 0.0;
    out[2] = pct(0.50);
    out[3] = pct(0.99);
    out[4] = (double)s->n_groups.load();
    out[5] = (double)s->peak.load();
    out[6] = (double)s->graph_steps.load();
    out[7] = (double)s->direct_steps.load();
  });
}
