/*
 * Matrix-free Lanczos recurrence for the ground energy of the transverse-field
 * Ising model on an Lx x Ly periodic square lattice (test infrastructure:
 * it pins the oracle's 2D Hamiltonian convention to the exact energy quoted by
 * the reference, examples/ising2d.jl:55, for the 5 x 5 lattice at h = 3; the
 * quoted value is the ferromagnetic coupling's, J = -1 here).  Never linked
 * into libnqcuda.
 *
 * H = -h Σ_p σx_p + J Σ_p (σz_p σz_{right(p)} + σz_p σz_{up(p)}) with the site
 * numbering of examples/ising2d.jl:16-26 (0-based: p = i + j Ly, right(p) =
 * ((i+1) mod Lx) + j Ly, up(p) = i + ((j+1) mod Ly) Ly).
 *
 * The global spin flip P = Π σx commutes with H and the ground state of this
 * model lies in its even sector (a positive-amplitude ground state of -H in
 * the σx basis; checked against dense diagonalisation on small lattices by the
 * tests).  Even-sector vectors are stored on the 2^(N-1) configurations whose
 * last site bit is 0: flipping the last site maps s to the complement of
 * s ^ bit(N-1), i.e. (~s) & (2^(N-1) - 1), with the same amplitude.
 *
 * The caller gets the tridiagonal Lanczos coefficients (alpha, beta) and takes
 * the lowest eigenvalue of the tridiagonal matrix; no reorthogonalisation is
 * done (the extreme Ritz value converges regardless; spurious copies only
 * repeat it).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static void tfim_matvec(int N, const int* bonds, int nb, double h, double J, const double* x, double* y,
                        int64_t dim, int z2) {
  const int last = N - 1;
  const int64_t mask = dim - 1;
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < dim; ++s) {
    double d = 0.0;
    for (int b = 0; b < nb; ++b) {
      const int p = bonds[2 * b], q = bonds[2 * b + 1];
      const int zp = (int)((s >> p) & 1), zq = (int)((s >> q) & 1);
      d += (zp == zq) ? J : -J;
    }
    double acc = d * x[s];
    const int nflip = z2 ? last : N;
    for (int i = 0; i < nflip; ++i) acc -= h * x[s ^ ((int64_t)1 << i)];
    if (z2) acc -= h * x[(~s) & mask];
    y[s] = acc;
  }
}

/* Runs `iters` Lanczos steps from a fixed pseudo-random start vector; fills
 * alpha[0..iters) and beta[0..iters-1).  Returns the number of steps done
 * (fewer if an invariant subspace is hit) or -1 if memory is short. */
int tfim2d_lanczos(int Lx, int Ly, double h, double J, int z2, int iters, double* alpha, double* beta) {
  const int N = Lx * Ly;
  if (N < 2 || N > 34) return -1;
  const int64_t dim = (int64_t)1 << (z2 ? N - 1 : N);
  int* bonds = (int*)malloc(sizeof(int) * 4 * N);
  int nb = 0;
  for (int i = 0; i < Lx; ++i)
    for (int j = 0; j < Ly; ++j) {
      const int p = i + j * Ly;
      bonds[2 * nb] = p; bonds[2 * nb + 1] = ((i + 1) % Lx) + j * Ly; ++nb;
      bonds[2 * nb] = p; bonds[2 * nb + 1] = i + ((j + 1) % Ly) * Ly; ++nb;
    }
  double* v0 = (double*)malloc(sizeof(double) * dim);
  double* v1 = (double*)malloc(sizeof(double) * dim);
  double* w = (double*)malloc(sizeof(double) * dim);
  if (!v0 || !v1 || !w) { free(v0); free(v1); free(w); free(bonds); return -1; }
  double nrm = 0.0;
#pragma omp parallel for reduction(+ : nrm)
  for (int64_t s = 0; s < dim; ++s) {
    uint64_t z = (uint64_t)s * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    z ^= z >> 29; z *= 0xBF58476D1CE4E5B9ull; z ^= z >> 32;
    v1[s] = 0.5 + (double)(z >> 11) * (1.0 / 9007199254740992.0);
    v0[s] = 0.0;
    nrm += v1[s] * v1[s];
  }
  nrm = sqrt(nrm);
#pragma omp parallel for
  for (int64_t s = 0; s < dim; ++s) v1[s] /= nrm;
  double b_prev = 0.0;
  int k = 0;
  for (; k < iters; ++k) {
    tfim_matvec(N, bonds, nb, h, J, v1, w, dim, z2);
    double a = 0.0;
#pragma omp parallel for reduction(+ : a)
    for (int64_t s = 0; s < dim; ++s) a += w[s] * v1[s];
    alpha[k] = a;
    double bb = 0.0;
#pragma omp parallel for reduction(+ : bb)
    for (int64_t s = 0; s < dim; ++s) {
      const double r = w[s] - a * v1[s] - b_prev * v0[s];
      w[s] = r;
      bb += r * r;
    }
    const double b = sqrt(bb);
    if (k + 1 < iters) beta[k] = b;
    if (b < 1e-14) { ++k; break; }
#pragma omp parallel for
    for (int64_t s = 0; s < dim; ++s) {
      v0[s] = v1[s];
      v1[s] = w[s] / b;
    }
    b_prev = b;
  }
  free(v0); free(v1); free(w); free(bonds);
  return k;
}
