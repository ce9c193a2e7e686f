/*
 * mdft_oracle.h -- CPU restatement of the Mini-MDFT excess-functional
 * convolution hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in mini_mdft_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it.  The product never links it.
 *
 * Parity status: the reference (Kokkos + kokkos-fft) cannot be compiled here,
 * so this restatement is pinned only by the reference's own known-answer
 * tests (Gauss-Legendre weight sum, Wigner-d quick returns and closed forms),
 * by numpy.fft cross-checks of its FFT conventions and by mathematical
 * identities; the end-to-end numbers are otherwise "parity unpinned" beyond
 * those checks.
 *
 * Every array is row-major ("LayoutRight"); complex numbers are two
 * interleaved doubles (re, im), as Kokkos::complex<double> is laid out.
 */
#ifndef MDFT_ORACLE_H
#define MDFT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mdft_oracle mdft_oracle;

/* Spatial grid + angular grid + orientation/projection map
 * (common/MDFT_Grid.hpp:184-238, :264-469;
 *  common/MDFT_OrientationProjectionTransform.hpp:55-148, :217-237). */
mdft_oracle* mdfto_create(int nx, int ny, int nz, double lx, double ly,
                          double lz, int mmax, int mrso);
void mdfto_destroy(mdft_oracle* o);
void mdfto_set_threads(mdft_oracle* o, int nthreads);

/* ints[0..]: nx ny nz mmax mrso ntheta nphi npsi no np npairs np_new nq */
void mdfto_info(const mdft_oracle* o, int* ints);

/* Host tables, copied out for tests. Sizes in the comments. */
void mdfto_kvectors(const mdft_oracle* o, double* kx, double* ky, double* kz);
void mdfto_angular(const mdft_oracle* o, double* thetaofntheta /*ntheta*/,
                   double* wthetaofntheta /*ntheta*/, double* w /*no*/);
void mdfto_opmap(const mdft_oracle* o, int* p /*(mmax+1)(2mmax+1)(mmax/mrso+1)*/,
                 int* m, int* mup, int* mu, int* mu2 /*np each*/,
                 double* wigner /*(ntheta,np)*/);

double mdfto_wigner_small_d(int m, int mu, int mup, double theta);
void mdfto_gauss_legendre(int n, double* x, double* w);
/* a,b: (5,13,13); c,d: (5,13) (common/MDFT_Rotation.hpp:22-85). */
void mdfto_rotation_coeffs(double* a, double* b, double* c, double* d);
/* R: complex (mmax+1, 2mmax+1, 2mmax+1); entries with |mup|>m or |khi|>m
 * are left untouched (the reference never writes them either). */
void mdfto_rotation_matrix(const double* q, int mmax, double* R);

/* Convolution set-up from a table in the Luc file layout
 * (common/IO/MDFT_ReadCLuc.hpp:40-120, common/MDFT_Convolution.hpp:106-313).
 * luc_index: 5 x np_luc ints (m, n, mu, nu, khi); luc: (np_luc, nq) complex.
 * Returns 0 on success, nonzero if nq is too small for the grid. */
int mdfto_set_luc(mdft_oracle* o, const int* luc_index, const double* luc,
                  int np_luc, int nq, double dq);
/* q_max the grid needs and the nq the Luc reader derives from it. */
double mdfto_qmax(const mdft_oracle* o);
int mdfto_nq_for_dq(const mdft_oracle* o, double dq);
void mdfto_gamma_p_map(const mdft_oracle* o, int* map /*(npairs,3)*/);
void mdfto_ia_map(const mdft_oracle* o, int* ia /*(np, mmax+1, 2mmax/mrso+1)*/);
void mdfto_mnmunukhi_q(const mdft_oracle* o, double* tab /*(np_new,nq) cplx*/);

/* The five hot-path stages (src/mini-mdft.hpp:137-183). */
void mdfto_delta_rho(const double* xi, double* delta_rho, size_t n, double rho0);
void mdfto_angl2proj(const mdft_oracle* o, const double* orient, double* proj);
void mdfto_proj2angl(const mdft_oracle* o, const double* proj, double* orient);
void mdfto_conv_execute(const mdft_oracle* o, double* proj);
double mdfto_delta_f(const double* xi, const double* vexc, const double* w,
                     double* delta_f, size_t nxyz, int no, double rho0,
                     double prefactor);

/* Batched unnormalised 3-D C2C FFT over the three trailing axes of
 * (batch, nx, ny, nz); sign -1 forward, +1 backward. */
void mdfto_fft3d(double* data, int batch, int nx, int ny, int nz, int sign);

/* Physical constants used by the energy prefactor
 * (common/MDFT_Constants.hpp, common/MDFT_Thermo.hpp:60,
 *  common/MDFT_Solvent.hpp:366-368). */
double mdfto_prefactor(double temperature, int mrso, double n0);

#ifdef __cplusplus
}
#endif
#endif
