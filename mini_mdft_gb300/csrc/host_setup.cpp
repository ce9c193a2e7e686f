// host_setup.cpp -- see host_setup.hpp.  Each function restates the
// constructor named beside it (paths relative to the Mini_MDFT root).
#include "host_setup.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <sstream>

namespace mdft {

namespace {
constexpr double kPi = 3.14159265358979323846;

// Factorials are exact in double up to 22!, which covers every index used
// for mmax <= 11 (MDFT_Wigner.hpp:20-54 tabulates the same values).
double fact(int k) {
  double f = 1.0;
  for (int i = 2; i <= k; ++i) f *= (double)i;
  return f;
}

// SpatialGrid::kproj (common/MDFT_Grid.hpp:222-238).
std::vector<double> kproj(int n, double d) {
  std::vector<double> k(n);
  int n1 = n / 2 + 1, n2 = (n - 1) / 2;
  for (int i = 0; i < n1; i++) k[i] = (double)i * d;
  for (int i = 0; i < n2; i++) k[i + n1] = (double)(i - n2) * d;
  return k;
}

inline int inv_index(int i, int n) { return i == 0 ? 0 : n - i; }
}  // namespace

// gauss_legendre (common/MDFT_Math_Utils.hpp:25-73): Newton iteration on
// P_n, weights normalised so that they sum to 1.
void gauss_legendre(int n, double* x, double* w) {
  int m = (n + 1) / 2;
  for (int i = 1; i <= m; ++i) {
    double xi = std::cos(kPi * (i - 0.25) / (n + 0.5));
    double dx = 1.0, pp = 0.0;
    for (int it = 0; it < 1000 && std::fabs(dx) > std::numeric_limits<double>::epsilon(); ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * xi * p2 - (j - 1) * p3) / j;
      }
      pp = n * (xi * p1 - p2) / (xi * xi - 1.0);
      dx = -p1 / pp;
      xi += dx;
    }
    x[i - 1] = xi;
    w[i - 1] = 1.0 / ((1.0 - xi * xi) * pp * pp);
    x[n - i] = -xi;
    w[n - i] = w[i - 1];
  }
}

namespace {
// 2 pi (a / na + b / nb) reduced exactly to [0, 2 pi) before the
// trigonometric functions (long double)
long double ang_angle(int a, int na, int b, int nb) {
  const long long num = (long long)(((a % na) + na) % na) * nb + (long long)(((b % nb) + nb) % nb) * na;
  const long long den = (long long)na * nb;
  const long double pi = 3.141592653589793238462643383279502884L;
  return 2.0L * pi * (long double)(num % den) / (long double)den;
}
}  // namespace

std::vector<double> ang_matrix_a2p(const Grid& g) {
  const int no = g.no, np = g.np;
  std::vector<double> T((size_t)2 * np * no, 0.0);
  const long double inv = 1.0L / (long double)(g.nphi * g.npsi);
  for (int ip = 0; ip < np; ++ip)
    for (int th = 0; th < g.ntheta; ++th) {
      const long double c = (long double)g.wigner[(size_t)th * np + ip] * g.wtheta[th] * g.fm[g.m[ip]] * inv;
      for (int f = 0; f < g.nphi; ++f)
        for (int s = 0; s < g.npsi; ++s) {
          const long double a = ang_angle(g.mup[ip] * f, g.nphi, g.mu2[ip] * s, g.npsi);
          const size_t k = ((size_t)th * g.nphi + f) * g.npsi + s;
          T[(size_t)(2 * ip) * no + k] = (double)(c * std::cos(a));
          T[(size_t)(2 * ip + 1) * no + k] = (double)(c * std::sin(a));
        }
    }
  return T;
}

std::vector<double> ang_matrix_p2a(const Grid& g) {
  const int no = g.no, np = g.np;
  std::vector<double> T((size_t)no * 2 * np, 0.0);
  for (int ip = 0; ip < np; ++ip)
    for (int th = 0; th < g.ntheta; ++th) {
      const long double c = (long double)g.wigner[(size_t)th * np + ip] * g.fm[g.m[ip]] * (g.mu2[ip] == 0 ? 1 : 2);
      for (int f = 0; f < g.nphi; ++f)
        for (int s = 0; s < g.npsi; ++s) {
          const long double a = ang_angle(g.mup[ip] * f, g.nphi, g.mu2[ip] * s, g.npsi);
          const size_t k = ((size_t)th * g.nphi + f) * g.npsi + s;
          T[k * 2 * np + 2 * ip] = (double)(c * std::cos(a));
          T[k * 2 * np + 2 * ip + 1] = (double)(c * std::sin(a));
        }
    }
  return T;
}

// wigner_small_d (common/MDFT_Wigner.hpp:63-130): Legendre recursion when
// one index is zero, the closed-form sum otherwise.
double wigner_small_d(int m, int mu, int mup, double theta) {
  if (std::abs(mu) > m || std::abs(mup) > m) return 0.0;
  if (m == 0) return 1.0;
  if (mu == 0 || mup == 0) {
    int mu0 = mu;
    double th0 = theta;
    if (mu == 0) {
      mu0 = mup;
      th0 = -theta;
    }
    double x = 1.0;
    if (mu0 < 0) {
      x = std::pow(-1.0, mu0);
      mu0 = -mu0;
    }
    double cc = std::cos(th0), pm1 = 0.0, pm = 1.0;
    for (int l = mu0 + 1; l <= m; ++l) {
      double pm2 = pm1;
      pm1 = pm;
      pm = (cc * (double)(2 * l - 1) * pm1 - (double)(l + mu0 - 1) * pm2) /
           (double)(l - mu0);
    }
    return x * std::pow(-1.0, mu0) * std::sqrt(fact(m - mu0) / fact(m + mu0)) *
           fact(2 * mu0) / (std::pow(2.0, mu0) * fact(mu0)) *
           std::pow(std::sin(th0), mu0) * pm;
  }
  double s = 0.0, cc = std::cos(0.5 * theta), ss = std::sin(0.5 * theta);
  for (int it = std::max(0, mu - mup); it <= std::min(m + mu, m - mup); ++it) {
    s += std::pow(-1.0, it) /
         (fact(m + mu - it) * fact(m - mup - it) * fact(it) * fact(it - mu + mup)) *
         std::pow(cc, 2 * m + mu - mup - 2 * it) * std::pow(ss, 2 * it - mu + mup);
  }
  return std::sqrt(fact(m + mu) * fact(m - mu) * fact(m + mup) * fact(m - mup)) * s;
}

Grid::Grid(int nx_, int ny_, int nz_, double lx_, double ly_, double lz_,
           int mmax_, int mrso_)
    : nx(nx_), ny(ny_), nz(nz_), lx(lx_), ly(ly_), lz(lz_), mmax(mmax_), mrso(mrso_) {
  // SpatialGrid ctor checks (MDFT_Grid.hpp:186-193).
  throw_if(lx <= 0 || ly <= 0 || lz <= 0, "The supercell cannot have negative length.");
  throw_if(nx <= 0 || ny <= 0 || nz <= 0, "The space is divided into grid nodes.");
  throw_if(nx > 4096 || ny > 4096 || nz > 4096, "grid axis longer than 4096", 4);
  // AngularGrid ctor checks (MDFT_Grid.hpp:266-268).
  throw_if(mmax <= 0, "The grid mmax must be greater than zero.");
  throw_if(mrso <= 0, "The grid molrotsymorder must be greater than zero.");
  throw_if(mmax > 10, "mmax above 10 is not supported", 4);
  kx = kproj(nx, 2.0 * kPi / lx);
  ky = kproj(ny, 2.0 * kPi / ly);
  kz = kproj(nz, 2.0 * kPi / lz);
  ntheta = mmax + 1;
  nphi = 2 * mmax + 1;
  K = mmax / mrso;
  npsi = 2 * K + 1;
  no = ntheta * nphi * npsi;
  np = 0;
  for (int mm = 0; mm <= mmax; ++mm)
    for (int a = -mm; a <= mm; ++a)
      for (int b = 0; b <= mm / mrso; ++b) np++;
  theta.resize(ntheta);
  wtheta.resize(ntheta);
  gauss_legendre(ntheta, theta.data(), wtheta.data());
  for (auto& t : theta) t = std::acos(t);
  // w(io) = wtheta * wphi * wpsi * 8 pi^2 (MDFT_Grid.hpp:308-376).
  w.resize(no);
  {
    double wphi = 1.0 / (double)nphi, wpsi = 1.0 / (double)(npsi * mrso);
    double qn = 8.0 * kPi * kPi;
    int io = 0;
    for (int it = 0; it < ntheta; ++it)
      for (int a = 0; a < nphi; ++a)
        for (int b = 0; b < npsi; ++b) w[io++] = wtheta[it] * wphi * wpsi * qn;
    double sw = 0;
    for (double v : w) sw += v;
    throw_if(std::fabs(sw - qn / mrso) > std::numeric_limits<double>::epsilon() * 100 * std::fabs(sw),
             "sum(m_w) != quadrature_norm/molrotsymorder");
  }
  // OrientationProjectionMap (MDFT_OrientationProjectionTransform.hpp:76-147).
  p.assign((size_t)(mmax + 1) * (2 * mmax + 1) * (K + 1), 0);
  m.resize(np);
  mup.resize(np);
  mu.resize(np);
  mu2.resize(np);
  int ip = 0;
  for (int mm = 0; mm <= mmax; ++mm)
    for (int a = -mm; a <= mm; ++a)
      for (int b = 0; b <= mm; b += mrso) {
        p[((size_t)mm * (2 * mmax + 1) + (a + mmax)) * (K + 1) + b / mrso] = ip;
        m[ip] = mm;
        mup[ip] = a;
        mu[ip] = b;
        mu2[ip] = b / mrso;
        ip++;
      }
  throw_if(ip != np, "ip after the loops must be equal to np");
  wigner.resize((size_t)ntheta * np);
  for (int q = 0; q < np; ++q)
    for (int it = 0; it < ntheta; ++it)
      wigner[(size_t)it * np + q] = wigner_small_d(m[q], mup[q], mu[q], theta[it]);
  fm.resize(mmax + 1);
  for (int mm = 0; mm <= mmax; ++mm) fm[mm] = std::sqrt(2.0 * (double)mm + 1.0);
  // ia_map (MDFT_Convolution.hpp:178-196).
  int n2 = 2 * mmax / mrso + 1;
  ia_map.assign((size_t)np * (mmax + 1) * n2, 0);
  int ia = 0;
  for (int q = 0; q < np; ++q) {
    int ikhi = mup[q];
    for (int in = std::abs(ikhi); in <= mmax; ++in)
      for (int inu2 = -in / mrso; inu2 <= in / mrso; ++inu2)
        ia_map[((size_t)q * (mmax + 1) + in) * n2 + inu2 + mmax / mrso] = ia++;
  }
  np_new = ia;
}

// q_max the convolution needs (MDFT_Convolution.hpp:214-231).
double Grid::qmax() const {
  double a = *std::max_element(kx.begin(), kx.end());
  double b = *std::max_element(ky.begin(), ky.end());
  double c = *std::max_element(kz.begin(), kz.begin() + (nz / 2 + 1));
  return std::sqrt(a * a + b * b + c * c);
}

RotationCoeffs::RotationCoeffs() {
  const int mm = kRotMmaxMax;
  double sqrtof[2 * kRotMmaxMax + 2] = {0};
  for (int i = 2; i < 14; ++i) sqrtof[i] = std::sqrt((double)(i - 1));
  const double sqrt2 = std::sqrt(2.0);
  std::fill(a, a + kRotL * kRotM * kRotM, 0.0);
  std::fill(b, b + kRotL * kRotM * kRotM, 0.0);
  std::fill(c, c + kRotL * kRotM, 0.0);
  std::fill(d, d + kRotL * kRotM, 0.0);
  for (int l = 2; l <= mm; ++l) {
    for (int mv = -l; mv <= l; ++mv) {
      for (int m1 = -l + 1; m1 < l; ++m1) {
        int idx = ((l - 2) * kRotM + (mv + mm)) * kRotM + (m1 + mm);
        a[idx] = sqrtof[l + mv + 1] * sqrtof[l - mv + 1] /
                 (sqrtof[l + m1 + 1] * sqrtof[l - m1 + 1]);
        b[idx] = sqrtof[l + mv + 1] * sqrtof[l + mv] /
                 (sqrt2 * sqrtof[l + m1 + 1] * sqrtof[l - m1 + 1]);
      }
      int m1 = l, idx = (l - 2) * kRotM + (mv + mm);
      c[idx] = sqrt2 * sqrtof[l + mv + 1] * sqrtof[l - mv + 1] /
               (sqrtof[l + m1 + 1] * sqrtof[l + m1]);
      d[idx] = sqrtof[l + mv + 1] * sqrtof[l + mv] /
               (sqrtof[l + m1 + 1] * sqrtof[l + m1]);
    }
  }
}

std::vector<int> gamma_p_map(int nx, int ny, int nz) {
  std::vector<unsigned char> isok((size_t)nx * ny * nz, 0);
  std::vector<int> out;
  for (int iz = 0; iz < nz / 2 + 1; ++iz) {
    int izm = inv_index(iz, nz);
    for (int iy = 0; iy < ny; ++iy) {
      int iym = inv_index(iy, ny);
      for (int ix = 0; ix < nx; ++ix) {
        int ixm = inv_index(ix, nx);
        size_t a = ((size_t)ix * ny + iy) * nz + iz;
        size_t b = ((size_t)ixm * ny + iym) * nz + izm;
        if (isok[a] && isok[b]) continue;
        out.push_back(ix);
        out.push_back(iy);
        out.push_back(iz);
        isok[a] = 1;
        isok[b] = 1;
      }
    }
  }
  return out;
}

namespace {
// deltaAbscissa (ReadCLuc.hpp:189-259): spacing of the first abscissas
// after the 17 header lines.
double delta_abscissa(const std::string& path) {
  std::ifstream f(path);
  std::string line;
  for (int i = 0; i < 17; ++i)
    throw_if(!std::getline(f, line), "Unexpected EOF while skipping lines in file: " + path, 3);
  double prev = 0, cur = 0;
  for (int i = 0; i < 2; ++i) {
    throw_if(!(f >> prev), "Error reading first abscissa in file: " + path, 3);
    f.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
    throw_if(!(f >> cur), "Error reading second abscissa in file: " + path, 3);
    f.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  }
  return cur - prev;
}
}  // namespace

LucTable read_luc_file(const std::string& path, int np_luc, double qmaxwanted) {
  {
    std::ifstream probe(path);
    throw_if(!probe.good(), "File: " + path + "does not exist.", 3);
  }
  throw_if(np_luc <= 0, "np_luc must be positive");
  LucTable t;
  t.np_luc = np_luc;
  t.dq = delta_abscissa(path);
  throw_if(!(t.dq > 0), "Non-positive abscissa step in file: " + path, 3);
  t.nq = (int)(qmaxwanted / t.dq + 0.5) + 2;
  t.index.assign((size_t)5 * np_luc, 0);
  t.tab.assign((size_t)np_luc * t.nq, std::complex<double>(0, 0));
  std::ifstream f(path);
  std::string dummy;
  for (int i = 0; i < 10; ++i) std::getline(f, dummy);
  std::string label;
  std::getline(f, label);
  for (int row = 0; row < 5; ++row) {
    throw_if(!(f >> label), "malformed projection index block in " + path, 3);
    for (int i = 0; i < np_luc; ++i)
      throw_if(!(f >> t.index[(size_t)row * np_luc + i]), "malformed projection index block in " + path, 3);
  }
  std::getline(f, label);
  std::getline(f, label);
  for (int iq = 0; iq < t.nq; ++iq) {
    std::string line;
    throw_if(!std::getline(f, line), "c(q) file has fewer q rows than the grid needs: " + path, 3);
    std::istringstream iss(line);
    double q;
    throw_if(!(iss >> q), "malformed q row in " + path, 3);
    for (int ip = 0; ip < np_luc; ++ip) {
      std::complex<double> z;
      throw_if(!(iss >> z), "malformed c(q) value in " + path, 3);
      t.tab[(size_t)ip * t.nq + iq] = z;
    }
    throw_if(q > qmaxwanted + 2.0 * t.dq, "q > qmaxwanted in file.", 3);
  }
  return t;
}

void write_luc_file(const std::string& path, const LucTable& t, const std::string& header) {
  throw_if(t.np_luc <= 0 || t.nq <= 0 || !(t.dq > 0), "invalid c(q) table extents");
  throw_if(t.index.size() != (size_t)5 * t.np_luc || t.tab.size() != (size_t)t.np_luc * t.nq,
           "c(q) table arrays do not match their extents");
  std::FILE* f = std::fopen(path.c_str(), "w");
  throw_if(!f, "cannot open " + path + " for writing", 3);
  std::string line;
  char buf[80];
  auto put = [&](const std::string& x) { std::fputs(x.c_str(), f); };
  put("# " + header + "\n");
  for (int i = 0; i < 9; ++i) put("#\n");
  put("# projection indices\n");
  const char* names[5] = {"m", "n", "mu", "nu", "khi"};
  for (int row = 0; row < 5; ++row) {
    line = names[row];
    for (int i = 0; i < t.np_luc; ++i) line += " " + std::to_string(t.index[(size_t)row * t.np_luc + i]);
    put(line + "\n");
  }
  put("# q  c(q) for each projection\n");
  for (int iq = 0; iq < t.nq; ++iq) {
    std::snprintf(buf, sizeof buf, "%.17g", iq * t.dq);
    line = buf;
    for (int ip = 0; ip < t.np_luc; ++ip) {
      const std::complex<double> z = t.tab[(size_t)ip * t.nq + iq];
      std::snprintf(buf, sizeof buf, " (%.17g,%.17g)", z.real(), z.imag());
      line += buf;
    }
    put(line + "\n");
  }
  const bool ok = std::ferror(f) == 0;
  throw_if(std::fclose(f) != 0 || !ok, "error writing " + path, 3);
}

std::vector<std::complex<double>> reorder_luc(const Grid& g, const LucTable& t, int nq) {
  const int mmax = g.mmax, mrso = g.mrso, K = g.K;
  const int npm = 2 * mmax / mrso + 1, m2 = 2 * mmax + 1;
  // 5-D projection index (ReadCLuc.hpp:88-103); untouched entries stay 0.
  std::vector<int> p5((size_t)(mmax + 1) * (mmax + 1) * npm * npm * m2, 0);
  auto P5 = [&](int a, int b, int c, int d, int e) -> int& {
    return p5[((((size_t)a * (mmax + 1) + b) * npm + c) * npm + d) * m2 + e];
  };
  for (int ip = 0; ip < t.np_luc; ++ip) {
    int im = t.index[0 * (size_t)t.np_luc + ip], in = t.index[1 * (size_t)t.np_luc + ip];
    int imu = t.index[2 * (size_t)t.np_luc + ip], inu = t.index[3 * (size_t)t.np_luc + ip];
    int ikhi = t.index[4 * (size_t)t.np_luc + ip];
    if (im < 0 || im > mmax || in < 0 || in > mmax) continue;
    int c = imu / mrso + K, d = inu / mrso + K, e = ikhi + mmax;
    if (c < 0 || c >= npm || d < 0 || d >= npm || e < 0 || e >= m2) continue;
    P5(im, in, c, d, e) = ip;
  }
  std::vector<std::complex<double>> out((size_t)g.np_new * nq);
  std::vector<int> n_new(g.np_new), nu_new(g.np_new), khi_new(g.np_new);
  int i = 0;
  for (int im = 0; im <= mmax; ++im)
    for (int ikhi = -im; ikhi <= im; ++ikhi)
      for (int imu2 = 0; imu2 <= im / mrso; ++imu2)
        for (int in = std::abs(ikhi); in <= mmax; ++in)
          for (int inu2 = -in / mrso; inu2 <= in / mrso; ++inu2) {
            n_new[i] = in;
            nu_new[i] = inu2 * mrso;
            khi_new[i] = ikhi;
            int ip = P5(im, in, imu2 + K, inu2 + K, ikhi + mmax);
            for (int iq = 0; iq < nq; ++iq) out[(size_t)i * nq + iq] = t.tab[(size_t)ip * t.nq + iq];
            i++;
          }
  throw_if(i != g.np_new, "internal: OZ coefficient count mismatch");
  // Sign fold (MDFT_Convolution.hpp:297-311).
  for (int q = 0; q < g.np_new; ++q) {
    double s = nu_new[q] < 0 ? std::pow(-1.0, (double)(khi_new[q] + nu_new[q]))
                             : std::pow(-1.0, (double)n_new[q]);
    for (int iq = 0; iq < nq; ++iq) out[(size_t)q * nq + iq] *= s;
  }
  return out;
}

}  // namespace mdft
