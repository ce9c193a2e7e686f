// handles.hpp -- the handle structures behind the opaque types of
// include/mdft_gb300.h, shared by capi.cu (the operator entry points) and
// server.cu (the job server, which drives the same plans).
#pragma once
#include <complex>
#include <vector>

#include "../../include/mdft_gb300.h"
#include "common.cuh"

struct mdft_grid_s {
  mdft::Grid g;
  explicit mdft_grid_s(const mdft::Grid& gg) : g(gg) {}
};

struct mdft_opt_s {
  mdft::Grid g;
  int prec;
  int device;
  int batch = 1;  // same-shape fields per call, stored back to back
  mdft::DevBuf coef_a2p, coef_p2a, tw_phi, tw_psi, ip_m, ip_mup, ip_mu2, pmap;
  mdft::DevBuf tc_bsl_a2p, tc_fexp_a2p, tc_bsl_p2a, tc_fexp_p2a;  // tensor-core path
  mdft::AngPlan plan{};
  explicit mdft_opt_s(const mdft::Grid& gg) : g(gg) {}
};

struct mdft_conv_s {
  mdft::Grid g;
  int prec;
  int device;
  int batch = 1;  // same-shape fields per call, p laid out (np, batch, nx, ny, nz)
  int npairs = 0, nq = 0;
  double dq = 0;
  std::vector<int> pair_list;                 // reference order (getter)
  std::vector<std::complex<double>> mnq;      // (np_new, nq) (getter)
  mdft::DevBuf pairs, kx, ky, kz, rot, pmap, ip_m, ip_mup, ip_mu2, ia_map, ctab, tw_x, tw_y, tw_z;
  mdft::DevBuf pinfo, palpha, ia_start, rtab, ceff;  // lane-per-pair OZ path
  // double-float form: the projections stay packed DF pairs between the
  // passes of execute() (needs the lane OZ path and one axis longer than 1)
  bool df_packed = false;
  mdft::OzPlan oz{};
  mdft::FftAxis ax{}, ay{}, az{};
  explicit mdft_conv_s(const mdft::Grid& gg) : g(gg) {}
};


namespace mdft {
namespace detail {
// The stages of one round trip on the first k fields of a batched plan
// (k <= batch; field layouts as for the plan's full batch, k fields long).
void angl2proj_fields(mdft_opt_s* h, const void* o, bool from_xi, double rho0, void* p, int k,
                      cudaStream_t s);
void proj2angl_fields(mdft_opt_s* h, const void* p, void* o, int k, cudaStream_t s);
void execute_fields(mdft_conv_s* h, void* p, int k, cudaStream_t s);
int current_device();
}  // namespace detail
}  // namespace mdft
