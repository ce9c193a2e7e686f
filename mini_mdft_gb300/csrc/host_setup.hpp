// host_setup.hpp -- host-side (FP64) set-up of the grids, the orientation /
// projection map, the rotation-recursion coefficients, the (q,-q) pair list
// and the OZ c(q) table.  These are the constructors of the reference's
// operators; they run once per handle on the CPU and their results are
// uploaded to the GPU.
#pragma once

#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

namespace mdft {

// Error type mirroring MDFT::Impl::Throw_If (common/MDFT_Asserts.hpp:15-28).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void throw_if(bool cond, const std::string& msg, int code = 1) {
  if (cond) throw Error(code, msg);
}

// SpatialGrid + AngularGrid + OrientationProjectionMap
// (common/MDFT_Grid.hpp:184-398, MDFT_OrientationProjectionTransform.hpp:55-148).
struct Grid {
  int nx = 0, ny = 0, nz = 0;
  double lx = 0, ly = 0, lz = 0;
  int mmax = 0, mrso = 0, ntheta = 0, nphi = 0, npsi = 0, no = 0, np = 0;
  int K = 0;  // mmax / mrso
  int np_new = 0;
  std::vector<double> kx, ky, kz;
  std::vector<double> theta, wtheta, w;  // thetaofntheta, wthetaofntheta, w
  std::vector<int> p;                    // (mmax+1, 2mmax+1, K+1)
  std::vector<int> m, mup, mu, mu2;      // (np)
  std::vector<double> wigner;            // (ntheta, np)
  std::vector<double> fm;                // (mmax+1)
  std::vector<int> ia_map;               // (np, mmax+1, 2mmax/mrso+1)

  Grid(int nx, int ny, int nz, double lx, double ly, double lz, int mmax,
       int mrso);
  long long N() const { return (long long)nx * ny * nz; }
  int pidx(int mm, int mupi, int mu2i) const {
    return p[((size_t)mm * (2 * mmax + 1) + mupi) * (K + 1) + mu2i];
  }
  double qmax() const;
};

// The angular transforms at one grid point are linear maps between the no
// real orientation values and the np complex projections; as dense real
// matrices (row-major, FP64):
//   angl2proj (MDFT_OrientationProjectionTransform.hpp:270-380): (2 np, no),
//     row 2 ip + c is Re (c = 0) / Im (c = 1) of p(ip), column
//     (theta nphi + phi) npsi + psi; entry
//     d(theta, ip) wtheta fm(m) / (nphi npsi) x cos / sin of
//     2 pi (mup phi / nphi + mu2 psi / npsi)  (the conjugated, unnormalised
//     rfft2 over (phi, psi) read at (mup mod nphi, mu2), contracted over theta);
//   proj2angl (:391-484): (no, 2 np), entry
//     w(mu2) d(theta, ip) fm(m) x cos / sin of the same angle, w = 1 for
//     mu2 = 0 and 2 otherwise (the synthesis over m, the scatter to FFT order
//     and the unnormalised C2R transform, which keeps the real part of the
//     kpsi = 0 column).
std::vector<double> ang_matrix_a2p(const Grid& g);
std::vector<double> ang_matrix_p2a(const Grid& g);

double wigner_small_d(int m, int mu, int mup, double theta);
void gauss_legendre(int n, double* x, double* w);

// RotationCoeffs (common/MDFT_Rotation.hpp:22-85): a,b (5,13,13), c,d (5,13).
constexpr int kRotMmaxMax = 6;
constexpr int kRotL = kRotMmaxMax - 1;
constexpr int kRotM = 2 * kRotMmaxMax + 1;
struct RotationCoeffs {
  double a[kRotL * kRotM * kRotM];
  double b[kRotL * kRotM * kRotM];
  double c[kRotL * kRotM];
  double d[kRotL * kRotM];
  RotationCoeffs();
};

// gamma_p_map (common/MDFT_Convolution.hpp:129-176): pair list of (ix,iy,iz)
// for the "q" member of each {q,-q}, in the reference's enumeration order.
std::vector<int> gamma_p_map(int nx, int ny, int nz);

// A c(q) table in the Luc layout (common/IO/MDFT_ReadCLuc.hpp:19-120).
struct LucTable {
  int np_luc = 0, nq = 0;
  double dq = 0;
  std::vector<int> index;                 // 5 x np_luc: m, n, mu, nu, khi
  std::vector<std::complex<double>> tab;  // (np_luc, nq)
};

// Reads the Luc text file (ReadCLuc.hpp:123-259) keeping the first
// int(qmaxwanted/dq + 0.5) + 2 rows.
LucTable read_luc_file(const std::string& path, int np_luc, double qmaxwanted);
// Writes a table in the same text layout (ReadCLuc.hpp:123-187 parses it):
// ten free lines (the first holds `header`), a label line, the five index
// rows m, n, mu, nu, khi, a label line, then one row 'q (re,im) ...' per q
// with q = iq dq; values printed with 17 significant digits (exact round trip).
void write_luc_file(const std::string& path, const LucTable& t, const std::string& header);

// Reorder + sign fold into mnmunukhi_q (np_new, nq_used)
// (common/MDFT_Convolution.hpp:239-311).
std::vector<std::complex<double>> reorder_luc(const Grid& g, const LucTable& t,
                                              int nq_used);

}  // namespace mdft
