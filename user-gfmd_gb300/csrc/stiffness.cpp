// Host-side Phi(q) table producer; see stiffness.h for the reference
// functions each part restates.
#include "stiffness.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <thread>

namespace gfmd {

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

void inv3(const double *m, double *r) {
  double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
               m[2] * (m[3] * m[7] - m[4] * m[6]);
  if (det == 0.0) throw std::runtime_error("singular surface cell");
  double id = 1.0 / det;
  r[0] = (m[4] * m[8] - m[5] * m[7]) * id;
  r[1] = (m[2] * m[7] - m[1] * m[8]) * id;
  r[2] = (m[1] * m[5] - m[2] * m[4]) * id;
  r[3] = (m[5] * m[6] - m[3] * m[8]) * id;
  r[4] = (m[0] * m[8] - m[2] * m[6]) * id;
  r[5] = (m[2] * m[3] - m[0] * m[5]) * id;
  r[6] = (m[3] * m[7] - m[4] * m[6]) * id;
  r[7] = (m[1] * m[6] - m[0] * m[7]) * id;
  r[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

void matvec3(const double *m, const double *v, double *r) {
  for (int i = 0; i < 3; i++) r[i] = m[3 * i] * v[0] + m[3 * i + 1] * v[1] + m[3 * i + 2] * v[2];
}

double parse_double(const std::vector<std::string> &tok, size_t &pos, const char *what,
                    double lo, double hi) {
  if (pos >= tok.size()) throw std::runtime_error(std::string("missing ") + what);
  const char *s = tok[pos].c_str();
  char *end;
  double v = std::strtod(s, &end);
  if (end == s) throw std::runtime_error(std::string("cannot convert ") + what + " '" + tok[pos] + "'");
  if (lo != hi && (v < lo || v > hi))
    throw std::runtime_error(std::string(what) + " out of range: '" + tok[pos] + "'");
  pos++;
  return v;
}

long parse_int(const std::vector<std::string> &tok, size_t &pos, const char *what, long lo,
               long hi) {
  if (pos >= tok.size()) throw std::runtime_error(std::string("missing ") + what);
  const char *s = tok[pos].c_str();
  char *end;
  long v = std::strtol(s, &end, 10);
  if (end == s) throw std::runtime_error(std::string("cannot convert ") + what + " '" + tok[pos] + "'");
  if (lo != hi && (v < lo || v > hi))
    throw std::runtime_error(std::string(what) + " out of range: '" + tok[pos] + "'");
  pos++;
  return v;
}

// ---- small dense complex matrices (row-major) ------------------------------

inline cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// C = A*B
void matmul(int n, const cplx *A, const cplx *B, cplx *C) {
  for (int i = 0; i < n; i++) {
    double cr[32], ci[32];
    for (int j = 0; j < n; j++) cr[j] = ci[j] = 0.0;
    for (int k = 0; k < n; k++) {
      double ar = A[i * n + k].re, ai = A[i * n + k].im;
      const cplx *b = B + k * n;
      for (int j = 0; j < n; j++) {
        cr[j] += ar * b[j].re - ai * b[j].im;
        ci[j] += ar * b[j].im + ai * b[j].re;
      }
    }
    for (int j = 0; j < n; j++) C[i * n + j] = {cr[j], ci[j]};
  }
}

// In-place inverse by Gauss-Jordan elimination with partial (row) pivoting.
bool invert(int n, cplx *A) {
  int perm[32];
  for (int c = 0; c < n; c++) {
    int p = c;
    double best = -1.0;
    for (int r = c; r < n; r++) {
      double m = A[r * n + c].re * A[r * n + c].re + A[r * n + c].im * A[r * n + c].im;
      if (m > best) { best = m; p = r; }
    }
    if (!(best > 0.0)) return false;
    perm[c] = p;
    if (p != c)
      for (int j = 0; j < n; j++) std::swap(A[c * n + j], A[p * n + j]);
    cplx piv = A[c * n + c];
    double d = 1.0 / (piv.re * piv.re + piv.im * piv.im);
    cplx pinv = {piv.re * d, -piv.im * d};
    A[c * n + c] = {1.0, 0.0};
    for (int j = 0; j < n; j++) A[c * n + j] = cmul(A[c * n + j], pinv);
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      cplx f = A[r * n + c];
      if (f.re == 0.0 && f.im == 0.0) continue;
      A[r * n + c] = {0.0, 0.0};
      for (int j = 0; j < n; j++) {
        cplx t = cmul(f, A[c * n + j]);
        A[r * n + j].re -= t.re;
        A[r * n + j].im -= t.im;
      }
    }
  }
  // undo the row interchanges as column interchanges, in reverse order
  for (int c = n - 1; c >= 0; c--) {
    int p = perm[c];
    if (p != c)
      for (int i = 0; i < n; i++) std::swap(A[i * n + c], A[i * n + p]);
  }
  return true;
}

// One step of the transfer-matrix recursion for a Hermitian positive definite
// A (row-major, lower triangle read):  X = -V A^{-1} V^H = -W^H W with
// A = L L^H (Cholesky) and W = L^{-1} V^H, about a third of the flops of an
// explicit inverse and two products.  L and W are n*n scratch.  Returns false
// when a pivot is not safely positive (below 1e-12 of its diagonal entry);
// the caller then takes the Gauss-Jordan path.
bool schur_step_chol(int n, const cplx *A, const cplx *V, cplx *X, cplx *L, cplx *W) {
  for (int j = 0; j < n; j++) {
    double djj = A[j * n + j].re;
    for (int k = 0; k < j; k++) djj -= L[j * n + k].re * L[j * n + k].re + L[j * n + k].im * L[j * n + k].im;
    if (!(djj > 1e-12 * std::fabs(A[j * n + j].re))) return false;
    const double ljj = std::sqrt(djj), inv = 1.0 / ljj;
    L[j * n + j] = {ljj, 0.0};
    for (int i = j + 1; i < n; i++) {
      double re = A[i * n + j].re, im = A[i * n + j].im;
      for (int k = 0; k < j; k++) {  // - L[i][k] conj(L[j][k])
        const cplx a = L[i * n + k], b = L[j * n + k];
        re -= a.re * b.re + a.im * b.im;
        im -= a.im * b.re - a.re * b.im;
      }
      L[i * n + j] = {re * inv, im * inv};
    }
  }
  // W = L^{-1} V^H, V^H[i][c] = conj(V[c][i])
  for (int i = 0; i < n; i++) {
    const double inv = 1.0 / L[i * n + i].re;
    for (int c = 0; c < n; c++) {
      double re = V[c * n + i].re, im = -V[c * n + i].im;
      for (int k = 0; k < i; k++) {
        const cplx a = L[i * n + k], w = W[k * n + c];
        re -= a.re * w.re - a.im * w.im;
        im -= a.re * w.im + a.im * w.re;
      }
      W[i * n + c] = {re * inv, im * inv};
    }
  }
  // X = -W^H W (Hermitian: upper triangle, mirrored)
  for (int i = 0; i < n; i++)
    for (int j = i; j < n; j++) {
      double re = 0.0, im = 0.0;
      for (int k = 0; k < n; k++) {  // conj(W[k][i]) W[k][j]
        const cplx a = W[k * n + i], b = W[k * n + j];
        re += a.re * b.re + a.im * b.im;
        im += a.re * b.im - a.im * b.re;
      }
      X[i * n + j] = {-re, i == j ? 0.0 : -im};
      if (j != i) X[j * n + i] = {-re, im};
    }
  return true;
}

}  // namespace

// ---- crystal surfaces -------------------------------------------------------

void CrystalSurface::set_cell(const double *c) {
  if (c[1] != 0.0 || c[3] != 0.0 || c[6] != 0.0 || c[7] != 0.0)
    throw std::runtime_error("cell must be aligned along x- and y-axis");
  std::memcpy(cell, c, sizeof(cell));
  inv3(cell, invcell);
}

// CrystalSurface::supercell(1, 1, nz) (src/main/crystal_surface.cpp:428-548),
// before any neighbour list exists.
void CrystalSurface::supercell_z(int nz) {
  double old_cell[9];
  std::memcpy(old_cell, cell, sizeof(cell));
  double nc[9];
  std::memcpy(nc, cell, sizeof(nc));
  nc[2] *= nz;
  nc[5] *= nz;
  nc[8] *= nz;
  nc[2] -= std::floor(nc[2] / nc[0]) * nc[0];
  nc[5] -= std::floor(nc[5] / nc[4]) * nc[4];
  set_cell(nc);
  std::vector<double> np(3 * nat * nz);
  for (int z = 0; z < nz; z++) {
    for (int i = 0; i < nat; i++) {
      int k = i + nat * z;
      double c[3] = {0.0, 0.0, (double)z}, d[3], p[3], s[3];
      matvec3(old_cell, c, d);
      for (int a = 0; a < 3; a++) p[a] = pos[3 * i + a] + d[a];
      matvec3(invcell, p, s);
      for (int a = 0; a < 3; a++) s[a] -= std::floor(s[a]);
      matvec3(cell, s, &np[3 * k]);
    }
  }
  nat *= nz;
  pos.swap(np);
}

void CrystalSurface::reverse_indices() {
  std::vector<double> np(pos.size());
  for (int i = 0; i < nat; i++)
    for (int a = 0; a < 3; a++) np[3 * i + a] = pos[3 * (nat - 1 - i) + a];
  pos.swap(np);
}

// set_cell_and_scale_atoms(a*cell): positions keep their scaled coordinates.
void CrystalSurface::scale_cell(double a) {
  double nc[9];
  for (int i = 0; i < 9; i++) nc[i] = a * cell[i];
  for (int i = 0; i < nat; i++) {
    double s[3];
    matvec3(invcell, &pos[3 * i], s);
    std::memcpy(&pos[3 * i], s, sizeof(s));
  }
  set_cell(nc);
  for (int i = 0; i < nat; i++) {
    double r[3];
    matvec3(cell, &pos[3 * i], r);
    std::memcpy(&pos[3 * i], r, sizeof(r));
  }
}

// compute_neighbor_list + identify_neighbor_shells
// (src/main/crystal_surface.cpp:166-258).  The search range uses the squared
// lattice-vector lengths exactly as the reference does.
void CrystalSurface::compute_neighbor_list(double rcut) {
  double lx = cell[0] * cell[0] + cell[3] * cell[3] + cell[6] * cell[6];
  double ly = cell[1] * cell[1] + cell[4] * cell[4] + cell[7] * cell[7];
  double lz = cell[2] * cell[2] + cell[5] * cell[5] + cell[8] * cell[8];
  int nx = (int)std::lrint(std::floor(rcut / lx)) + 1;
  int ny = (int)std::lrint(std::floor(rcut / ly)) + 1;
  int nz = (int)std::lrint(std::floor(rcut / lz)) + 1;
  neigh.clear();
  for (int i = 0; i < nat; i++) {
    for (int j = 0; j < nat; j++) {
      for (int x = -nx; x <= nx; x++) {
        for (int y = -ny; y <= ny; y++) {
          for (int z = -nz; z <= nz; z++) {
            if (i == j && x == 0 && y == 0 && z == 0) continue;
            double d[3] = {(double)x, (double)y, (double)z}, cd[3];
            matvec3(cell, d, cd);
            LatticeNeighbor n;
            for (int a = 0; a < 3; a++) n.r[a] = pos[3 * i + a] - pos[3 * j + a] - cd[a];
            n.rnorm = std::sqrt(n.r[0] * n.r[0] + n.r[1] * n.r[1] + n.r[2] * n.r[2]);
            if (n.rnorm < rcut) {
              n.i = i;
              n.j = j;
              n.x = x;
              n.y = y;
              n.ab = z;
              n.shell = -1;
              neigh.push_back(n);
            }
          }
        }
      }
    }
  }
  std::vector<double> shells;
  for (auto &n : neigh) {
    bool found = false;
    for (double r : shells)
      if (std::abs(n.rnorm - r) < 0.01) { found = true; break; }
    if (!found) shells.push_back(n.rnorm);
  }
  std::sort(shells.begin(), shells.end());
  for (auto &n : neigh)
    for (size_t k = 0; k < shells.size(); k++)
      if (std::abs(n.rnorm - shells[k]) < 0.01) { n.shell = (int)k; break; }
}

// ---- the ft kernel with pair-potential force constants ---------------------

StiffnessKernel *StiffnessKernel::create(const std::vector<std::string> &tok, size_t &pos) {
  if (pos >= tok.size()) throw std::runtime_error("missing stiffness kernel keyword");
  const std::string kw = tok[pos++];
  if (kw == "sc100" || kw == "fcc100") return create_analytic(kw, tok, pos);
  if (kw == "isotropic" || kw == "nonperiodic") return create_continuum(kw, tok, pos);
  if (kw != "ft")
    throw std::runtime_error("stiffness kernel '" + kw +
                             "' has no table producer here; pass its table to gfmd_set_phi");
  StiffnessKernel *k = new StiffnessKernel();
  try {
    k->name_ = "ft";
    // crystal surface (crystal_surface_factory, src/main/crystal_surface.cpp:696-725)
    if (pos >= tok.size()) throw std::runtime_error("missing crystal surface");
    const std::string sname = tok[pos++];
    CrystalSurface &s = k->surf_;
    s.name = sname;
    const double r2 = std::sqrt(2.0), r3 = std::sqrt(3.0);
    if (sname == "sc100") {
      const double c[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
      s.set_cell(c);
      s.nat = 1;
      s.pos = {0, 0, 0};
    } else if (sname == "fcc100") {
      const double c[9] = {1, 0, 0.5, 0, 1, 0.5, 0, 0, 1.0 / r2};
      s.set_cell(c);
      s.nat = 1;
      s.pos = {0, 0, 0};
    } else if (sname == "fcc111") {
      const double c[9] = {1, 0, 0.5, 0, r3, 1.0 / (2.0 * r3), 0, 0, std::sqrt(2.0 / 3.0)};
      s.set_cell(c);
      s.nat = 2;
      s.pos.assign(6, 0.0);
      const double sp[3] = {0.5, 0.5, 0.0};
      matvec3(s.cell, sp, &s.pos[3]);
    } else {
      throw std::runtime_error("could not find crystal surface '" + sname + "'");
    }
    double a = parse_double(tok, pos, "lattice constant", 0, 100);
    int nu = (int)parse_int(tok, pos, "number of lattice cells", 1, 100);
    if (nu > 1) {
      s.supercell_z(nu);
      s.reverse_indices();
    }
    s.scale_cell(a);

    // force constants (force_constants_factory, src/main/force_constants.cpp:113-164)
    if (pos >= tok.size()) throw std::runtime_error("missing interaction model");
    const std::string fc = tok[pos++];
    if (fc != "pair-potential")
      throw std::runtime_error("interaction model '" + fc + "' is not available here");
    s.compute_neighbor_list(2.01 * std::max(s.cell[0], s.cell[4]));
    if (pos >= tok.size()) throw std::runtime_error("missing number of interacting neighbors");
    std::string nks = tok[pos];
    bool x = !nks.empty() && nks.back() == 'x';
    if (x) nks.pop_back();
    {
      char *end;
      long nk = std::strtol(nks.c_str(), &end, 10);
      if (end == nks.c_str()) throw std::runtime_error("cannot convert neighbor shell count");
      if (nk < 0 || nk > 3) throw std::runtime_error("at most 3 neighbor shells are supported");
      pos++;
      for (long i = 0; i < nk; i++) {
        k->k_[i] = parse_double(tok, pos, "spring constant", 0, 0);
        if (x) k->kappa_[i] = parse_double(tok, pos, "spring constant", 0, 0);
      }
    }
    // optional keywords: `linf` (fc_pair_potential.cpp:99-132), `height` (ft_stiffness.cpp:85-99)
    k->linf_.assign(s.nat, 0.0);
    bool found = true;
    while (pos + 1 < tok.size() && found) {
      found = false;
      if (tok[pos] == "linf") {
        pos++;
        int nl = (int)parse_int(tok, pos, "number of layers", 0, 0);
        if (nl != s.nat) throw std::runtime_error("linf: number of layers must match the surface cell");
        double sum = 0.0;
        for (int i = 0; i < nl; i++) {
          k->linf_[i] = parse_double(tok, pos, "linf", 0, 0);
          sum += k->linf_[i];
        }
        if (std::abs(sum) > 1e-12) throw std::runtime_error("linear force contributions must sum to zero");
        found = true;
      } else if (tok[pos] == "height") {
        pos++;
        k->height_ = (int)parse_int(tok, pos, "height", 0, 0);
        found = true;
      }
    }
    k->dim_ = 3 * s.nat;
    k->pre_compute();
  } catch (...) {
    delete k;
    throw;
  }
  return k;
}

// ---- the continuum styles ----------------------------------------------------

// IsotropicStiffnessKernel (src/stiffness_kernels/isotropic_stiffness.cpp:43-87):
//   isotropic nu mu gamma      (height 1 when 0 < gamma < 1e6, else 0)
// NonperiodicStiffnessKernel (src/stiffness_kernels/nonperiodic_stiffness.cpp:44-102):
//   nonperiodic nu mu          (height 1)
StiffnessKernel *StiffnessKernel::create_continuum(const std::string &kw, const std::vector<std::string> &tok,
                                                   size_t &pos) {
  StiffnessKernel *k = new StiffnessKernel();
  try {
    k->name_ = kw;
    k->nu_ = 1;
    k->dim_ = 3;
    k->poisson_ = parse_double(tok, pos, "Poisson number", 0, 0);
    k->shear_ = parse_double(tok, pos, "shear modulus", 0, 0);
    if (kw == "isotropic") {
      k->kind_ = kIsotropic;
      k->gamma_ = parse_double(tok, pos, "gamma", 0, 0);
      k->height_ = (k->gamma_ > 0.0 && k->gamma_ < 1e6) ? 1 : 0;
    } else {
      k->kind_ = kNonperiodic;
      k->height_ = 1;
    }
  } catch (...) {
    delete k;
    throw;
  }
  return k;
}

// Surface Green's function of an isotropic elastic half-space in Fourier
// space (q in radians per grid spacing), inverted to a stiffness; at q = 0 the
// finite-box compliance diag((1/2 + 1/(2(1-nu))) xprd, same, xprd)/(gamma pi).
// Follows IsotropicStiffnessKernel::get_stiffness_matrix
// (isotropic_stiffness.cpp:91-146); the shear modulus is mu, the Poisson
// number nu, and 2 - 1/alpha = 2 nu, 1 - 1/alpha = 2 nu - 1 with
// alpha = 1/(2(1-nu)).
bool StiffnessKernel::isotropic(double qx, double qy, double xprd, double yprd, cplx *phi) const {
  (void)yprd;
  const double alpha = 1.0 / (2.0 * (1.0 - poisson_));
  for (int i = 0; i < 9; i++) phi[i] = {0.0, 0.0};
  if (std::fabs(qx) <= 1e-6 && std::fabs(qy) <= 1e-6) {
    const double cz = xprd / (gamma_ * kPi);
    phi[0].re = (alpha + 0.5) * cz;
    phi[4].re = phi[0].re;
    phi[8].re = cz;
    return invert(3, phi);
  }
  const double q2 = qx * qx + qy * qy, q = std::sqrt(q2);
  const double mu = shear_, nu = poisson_;
  const double inplane = 2.0 * nu / (2.0 * mu * q * q2);  // (2 - 1/alpha) / (2 mu q^3)
  const double normal = (2.0 * nu - 1.0) / (2.0 * mu * q2);  // (1 - 1/alpha) / (2 mu q^2)
  phi[0].re = 1.0 / (mu * q) - qx * qx * inplane;
  phi[4].re = 1.0 / (mu * q) - qy * qy * inplane;
  phi[8].re = 1.0 / (2.0 * mu * alpha * q);
  phi[1].re = phi[3].re = -qx * qy * inplane;
  phi[2].im = -qx * normal;
  phi[5].im = -qy * normal;
  phi[6].im = qx * normal;
  phi[7].im = qy * normal;
  return invert(3, phi);
}

namespace {

// Y * ln(X + r), r = |(X, Y)|, zero on the line Y = 0; for X < 0 through
// X + r = Y^2 / (r - X), which has no cancellation.
double y_log_x_plus_r(double Y, double X) {
  if (Y == 0.0) return 0.0;
  const double r = std::sqrt(X * X + Y * Y);
  return Y * (X >= 0.0 ? std::log(X + r) : std::log(Y * Y / (r - X)));
}

// X * atan(Y / X) + Y/2 * ln(X^2 + Y^2): an antiderivative in X and Y of X / r^2.
double prim_x_over_r2(double X, double Y) {
  const double r2 = X * X + Y * Y;
  double v = X == 0.0 ? 0.0 : X * std::atan(Y / X);
  if (Y != 0.0) v += 0.5 * Y * std::log(r2);
  return v;
}

}  // namespace

// Displacements at the surface of an isotropic half-space (shear modulus mu,
// Poisson number nu) under a unit force spread uniformly over one grid cell
// [-dx/2, dx/2] x [-dy/2, dy/2], at the grid point offset (i dx, j dy).  The
// point-force solutions of Boussinesq (normal) and Cerruti (tangential), in
// the reference's orientation (z and the normal force positive away from the
// solid), are, with c = (1 - 2 nu) / (4 pi mu) and r = |(x, y)|:
//   normal force P:       u_x = c P x/r^2,  u_y = c P y/r^2,
//                         u_z = (1 - nu) P / (2 pi mu r)
//   tangential force Q_x: u_x = Q_x/(2 pi mu) ((1 - nu)/r + nu x^2/r^3),
//                         u_y = Q_x/(2 pi mu) nu x y/r^3,  u_z = -c Q_x x/r^2
// (Q_y by symmetry).  Their integrals over the cell are closed-form corner
// sums of antiderivatives F with d2F/dxdy = integrand:
//   1/r -> x ln(y + r) + y ln(x + r),   x/r^2 -> x atan(y/x) + y/2 ln r^2,
//   x^2/r^3 -> y ln(x + r),             x y/r^3 -> -r.
// The reference integrates the same solutions over two triangles per cell
// (sq_uniform_PQ, src/stiffness_kernels/li_berger.cpp:453-459, after Li and
// Berger, J. Elasticity 63, 137 (2001)); both are exact up to rounding.
void StiffnessKernel::nonperiodic_green(int i, int j, double dx, double dy, double *G) const {
  const double mu = shear_, nu = poisson_;
  const double a = 0.5 * dx, b = 0.5 * dy;
  const double x[2] = {i * dx - a, i * dx + a}, y[2] = {j * dy - b, j * dy + b};
  double inv_r = 0, x_r2 = 0, y_r2 = 0, xx_r3 = 0, yy_r3 = 0, xy_r3 = 0;
  for (int cx = 0; cx < 2; cx++)
    for (int cy = 0; cy < 2; cy++) {
      const double sgn = (cx == cy) ? 1.0 : -1.0;
      const double X = x[cx], Y = y[cy];
      const double xl = y_log_x_plus_r(X, Y), yl = y_log_x_plus_r(Y, X);  // X ln(Y+r), Y ln(X+r)
      inv_r += sgn * (xl + yl);
      x_r2 += sgn * prim_x_over_r2(X, Y);
      y_r2 += sgn * prim_x_over_r2(Y, X);
      xx_r3 += sgn * yl;
      yy_r3 += sgn * xl;
      xy_r3 -= sgn * std::sqrt(X * X + Y * Y);
    }
  // unit total force: traction 1/(dx dy) over the cell
  const double t = 1.0 / (dx * dy);
  const double c = (1.0 - 2.0 * nu) / (4.0 * kPi * mu) * t, s = t / (2.0 * kPi * mu);
  // columns: traction x, y, z
  G[0] = s * ((1.0 - nu) * inv_r + nu * xx_r3);
  G[3] = s * nu * xy_r3;
  G[6] = -c * x_r2;
  G[1] = s * nu * xy_r3;
  G[4] = s * ((1.0 - nu) * inv_r + nu * yy_r3);
  G[7] = -c * y_r2;
  G[2] = c * x_r2;
  G[5] = c * y_r2;
  G[8] = (1.0 - nu) * s * inv_r;
}

// ---- the analytic styles -----------------------------------------------------

// SC100StiffnessKernel (src/stiffness_kernels/sc100_stiffness.cpp:137-160):
//   sc100 [height N]
// FCC100StiffnessKernel (src/stiffness_kernels/fcc100_stiffness.cpp:57-242):
//   fcc100 [x] nu k1 [kappa1] [k2 [kappa2] k3 [kappa3]] {height N | linf l1..l_nu |
//          normal +-1 | mulphase m}
// (one spring constant for nu = 1, three otherwise; kappas with `x`).
StiffnessKernel *StiffnessKernel::create_analytic(const std::string &kw, const std::vector<std::string> &tok,
                                                  size_t &pos) {
  StiffnessKernel *k = new StiffnessKernel();
  try {
    k->name_ = kw;
    if (kw == "sc100") {
      k->kind_ = kSC100;
      k->nu_ = 1;
      if (pos + 1 < tok.size() && tok[pos] == "height") {
        pos++;
        k->height_ = (int)parse_int(tok, pos, "height", 0, 0);
      }
    } else {
      k->kind_ = kFCC100;
      if (pos >= tok.size()) throw std::runtime_error("fcc100: expected the number of interacting neighbors");
      bool x = false;
      if (!tok[pos].empty() && tok[pos].back() == 'x') {
        x = true;
        pos++;
      }
      k->nu_ = (int)parse_int(tok, pos, "number of layers", 1, 4);
      const int nk = k->nu_ == 1 ? 1 : 3;
      for (int i = 0; i < nk; i++) {
        k->k_[i] = parse_double(tok, pos, "spring constant", 0, 0);
        if (x) k->kappa_[i] = parse_double(tok, pos, "spring constant", 0, 0);
      }
      k->linf_.assign(k->nu_, 0.0);
      bool found = true;
      while (pos + 1 < tok.size() && found) {
        found = false;
        if (tok[pos] == "height") {
          pos++;
          k->height_ = (int)parse_int(tok, pos, "height", 0, 0);
          found = true;
        } else if (tok[pos] == "linf") {
          pos++;
          double sum = 0.0;
          for (int i = 0; i < k->nu_; i++) {
            k->linf_[i] = parse_double(tok, pos, "linf", 0, 0);
            sum += k->linf_[i];
          }
          if (std::fabs(sum) > 1e-12) throw std::runtime_error("linear force contributions must sum to zero");
          found = true;
        } else if (tok[pos] == "normal") {
          pos++;
          k->z_ = (int)parse_int(tok, pos, "surface normal", -1, 1);
          if (k->z_ != 1 && k->z_ != -1) throw std::runtime_error("surface normal must be +1 or -1");
          found = true;
        } else if (tok[pos] == "mulphase") {
          pos++;
          parse_double(tok, pos, "mulphase", 0, 0);  // parsed, not used by the matrices
          found = true;
        }
      }
    }
    k->dim_ = 3 * k->nu_;
  } catch (...) {
    delete k;
    throw;
  }
  return k;
}

void StiffnessKernel::analytic_layers(double qx, double qy, cplx *D, double *xc, double *yc) const {
  const int nu = nu_;
  auto B = [&](int r, int c) { return D + 9 * (size_t)(r * (nu + 1) + c); };
  for (size_t i = 0; i < 9 * (size_t)(nu + 1) * (nu + 1); i++) D[i] = {0.0, 0.0};
  for (int i = 0; i < nu; i++) xc[i] = yc[i] = 0.0;
  auto re = [](cplx *M, int a, int b) -> double & { return M[3 * a + b].re; };
  auto im = [](cplx *M, int a, int b) -> double & { return M[3 * a + b].im; };
  const double cx = std::cos(qx), cy = std::cos(qy), sx = std::sin(qx), sy = std::sin(qy);
  if (kind_ == kSC100) {
    // SC100StiffnessKernel::get_per_layer_dynamical_matrices (sc100_stiffness.cpp:167-227)
    cplx *U0 = B(0, 0), *U = B(0, 1), *V0 = B(1, 0), *V = B(1, 1);
    re(U, 0, 0) = 6 - 2 * cx * (1 + cy);
    re(U, 1, 1) = 6 - 2 * cy * (1 + cx);
    re(U, 2, 2) = 6;
    re(U, 0, 1) = 2 * sx * sy;
    re(U, 1, 0) = 2 * sx * sy;
    re(U0, 0, 0) = 5 - 2 * cx * (1 + cy);
    re(U0, 1, 1) = 5 - 2 * cy * (1 + cx);
    re(U0, 2, 2) = 3;
    re(U0, 0, 1) = 2 * sx * sy;
    re(U0, 1, 0) = 2 * sx * sy;
    re(V, 0, 0) = -cx;
    re(V, 1, 1) = -cy;
    re(V, 2, 2) = -1 - cx - cy;
    im(V, 0, 2) = sx;
    im(V, 1, 2) = sy;
    im(V, 2, 0) = sx;
    im(V, 2, 1) = sy;
    std::memcpy(V0, V, 9 * sizeof(cplx));  // pair potential: V0 = V
    return;
  }
  // FCC100StiffnessKernel::get_per_layer_dynamical_matrices (fcc100_stiffness.cpp:276-480),
  // the equations of the reference's PRB appendix (A12-A30) in its arithmetic order
  const double cx2 = std::cos(qx / 2), cy2 = std::cos(qy / 2), sx2 = std::sin(qx / 2), sy2 = std::sin(qy / 2);
  const double sqrt2 = std::sqrt(2.0);
  const double *k = k_, *kap = kappa_;
  const int z = z_;
  cplx *U0 = B(0, 0), *U = B(0, nu), *V0 = B(1, 0), *V = B(1, nu), *W = B(2 < nu + 1 ? 2 : 0, nu);
  // nearest neighbours (A12-A17)
  re(U, 0, 0) = k[0] * (4 - 2 * cx) + kap[0] * (8 - 2 * cy);
  re(U, 1, 1) = k[0] * (4 - 2 * cy) + kap[0] * (8 - 2 * cx);
  re(U, 2, 2) = k[0] * 4 + kap[0] * (8 - 2 * cx - 2 * cy);
  re(U0, 0, 0) = re(U, 0, 0) - k[0] * 1 - kap[0] * 3;
  re(U0, 1, 1) = re(U, 1, 1) - k[0] * 1 - kap[0] * 3;
  re(U0, 2, 2) = re(U, 2, 2) - k[0] * 2 - kap[0] * 2;
  re(V, 0, 0) = -k[0] * cx2 * cy2 - kap[0] * 3 * cx2 * cy2;
  re(V, 1, 1) = -k[0] * cx2 * cy2 - kap[0] * 3 * cx2 * cy2;
  re(V, 2, 2) = -k[0] * 2 * cx2 * cy2 - kap[0] * 2 * cx2 * cy2;
  re(V, 0, 1) = k[0] * sx2 * sy2 - kap[0] * sx2 * sy2;
  im(V, 0, 2) = z * (k[0] * sqrt2 * sx2 * cy2 - kap[0] * sqrt2 * sx2 * cy2);
  im(V, 1, 2) = z * (k[0] * sqrt2 * cx2 * sy2 - kap[0] * sqrt2 * cx2 * sy2);
  re(V, 1, 0) = k[0] * sx2 * sy2 - kap[0] * sx2 * sy2;
  im(V, 2, 0) = z * (k[0] * sqrt2 * sx2 * cy2 - kap[0] * sqrt2 * sx2 * cy2);
  im(V, 2, 1) = z * (k[0] * sqrt2 * cx2 * sy2 - kap[0] * sqrt2 * cx2 * sy2);
  if (nu >= 2) {
    // second and third neighbours, a full cell vertically (A21-A30)
    cplx *U1 = B(0, 1);
    double u2[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    u2[0] = k[1] * (2 - 2 * cx * cy) + kap[1] * (4 - 2 * cx * cy) + k[2] * 8 + kap[2] * 16;
    u2[4] = k[1] * (2 - 2 * cx * cy) + kap[1] * (4 - 2 * cx * cy) + k[2] * 8 + kap[2] * 16;
    u2[8] = k[1] * 2 + kap[1] * (4 - 4 * cx * cy) + k[2] * 8 + kap[2] * 16;
    u2[1] = k[1] * 2 * sx * sy - kap[1] * 2 * sx * sy;
    u2[3] = k[1] * 2 * sx * sy - kap[1] * 2 * sx * sy;
    for (int a = 0; a < 9; a++) {
      U0[a].re += u2[a];
      U[a].re += u2[a];
    }
    std::memcpy(U1, U, 9 * sizeof(cplx));
    re(U0, 0, 0) -= kap[1] + k[2] * 4 + kap[2] * 8;
    re(U0, 1, 1) -= kap[1] + k[2] * 4 + kap[2] * 8;
    re(U0, 2, 2) -= k[1] + k[2] * 4 + kap[2] * 8;
    re(U1, 0, 0) -= kap[1] + k[2] * 2 / 3 + kap[2] * 10 / 3;
    re(U1, 1, 1) -= kap[1] + k[2] * 2 / 3 + kap[2] * 10 / 3;
    re(U1, 2, 2) -= k[1] + k[2] * 8 / 3 + kap[2] * 4 / 3;
    re(V, 0, 0) += -k[2] * 1 / 3 * cx2 * cy2 * (-10 + 18 * cx + 2 * cy) -
                   kap[2] * 1 / 3 * cx2 * cy2 * (-14 + 6 * cx + 22 * cy);
    re(V, 1, 1) += -k[2] * 1 / 3 * cx2 * cy2 * (-10 + 2 * cx + 18 * cy) -
                   kap[2] * 1 / 3 * cx2 * cy2 * (-14 + 22 * cx + 6 * cy);
    re(V, 2, 2) += -k[2] * 2 / 3 * cx2 * cy2 * (-2 + 2 * (cx + cy)) -
                   kap[2] * 2 / 3 * cx2 * cy2 * (-10 + 10 * (cx + cy));
    re(V, 0, 1) += -k[2] * (-2 - 2 * (cx + cy)) * sx2 * sy2 - kap[2] * (2 + 2 * (cx + cy)) * sx2 * sy2;
    im(V, 0, 2) += z * (-k[2] * 1 / 3 * sqrt2 * cy2 * (-2 - 2 * (3 * cx + cy)) * sx2 -
                        kap[2] * 1 / 3 * sqrt2 * cy2 * (2 + 2 * (3 * cx + cy)) * sx2);
    im(V, 1, 2) += z * (-k[2] * 1 / 3 * sqrt2 * cx2 * (-2 - 2 * (cx + 3 * cy)) * sy2 -
                        kap[2] * 1 / 3 * sqrt2 * cx2 * (2 + 2 * (cx + 3 * cy)) * sy2);
    re(V, 1, 0) += -k[2] * (-2 - 2 * (cx + cy)) * sx2 * sy2 - kap[2] * (2 + 2 * (cx + cy)) * sx2 * sy2;
    im(V, 2, 0) += z * (-k[2] * 1 / 3 * sqrt2 * cy2 * (-2 - 2 * (3 * cx + cy)) * sx2 -
                        kap[2] * 1 / 3 * sqrt2 * cy2 * (2 + 2 * (3 * cx + cy)) * sx2);
    im(V, 2, 1) += z * (-k[2] * 1 / 3 * sqrt2 * cx2 * (-2 - 2 * (cx + 3 * cy)) * sy2 -
                        kap[2] * 1 / 3 * sqrt2 * cx2 * (2 + 2 * (cx + 3 * cy)) * sy2);
    re(W, 0, 0) = -kap[1] - k[2] * 2 / 3 * cx - kap[2] * (4 * cx / 3 + 2 * cy);
    re(W, 1, 1) = -kap[1] - k[2] * 2 / 3 * cy - kap[2] * (2 * cx + 4 * cy / 3);
    re(W, 2, 2) = -k[1] - k[2] * 4 / 3 * (cx + cy) - kap[2] * 2 / 3 * (cx + cy);
    im(W, 0, 2) = z * (k[2] * 2 / 3 * sqrt2 * sx - kap[2] * 2 / 3 * sqrt2 * sx);
    im(W, 1, 2) = z * (k[2] * 2 / 3 * sqrt2 * sy - kap[2] * 2 / 3 * sqrt2 * sy);
    im(W, 2, 0) = z * (k[2] * 2 / 3 * sqrt2 * sx - kap[2] * 2 / 3 * sqrt2 * sx);
    im(W, 2, 1) = z * (k[2] * 2 / 3 * sqrt2 * sy - kap[2] * 2 / 3 * sqrt2 * sy);
  }
  // pair potential: the per-layer V, W equal the bulk ones; U2, U3 too
  std::memcpy(V0, V, 9 * sizeof(cplx));
  if (nu > 1) {
    std::memcpy(B(1, 1), V, 9 * sizeof(cplx));
    std::memcpy(B(2, 0), W, 9 * sizeof(cplx));
    std::memcpy(B(2, 1), W, 9 * sizeof(cplx));
  }
  if (nu > 2) {
    std::memcpy(B(0, 2), U, 9 * sizeof(cplx));
    std::memcpy(B(1, 2), V, 9 * sizeof(cplx));
    std::memcpy(B(2, 2), W, 9 * sizeof(cplx));
  }
  if (nu > 3) {
    std::memcpy(B(0, 3), U, 9 * sizeof(cplx));
    std::memcpy(B(1, 3), V, 9 * sizeof(cplx));
    std::memcpy(B(2, 3), W, 9 * sizeof(cplx));
  }
  if (nu == 2 || nu == 4) xc[1] = yc[1] = 0.5;
  if (nu == 4) xc[3] = yc[3] = 0.5;
}

// FCPairPotential::offsite: D = -k e(x)e - kappa (1 - e(x)e).
void StiffnessKernel::offsite(const LatticeNeighbor &n, double *D) const {
  double e[3] = {n.r[0] / n.rnorm, n.r[1] / n.rnorm, n.r[2] / n.rnorm};
  double k = 0.0, kap = 0.0;
  if (n.shell < 3) {
    k = k_[n.shell];
    kap = kappa_[n.shell];
  }
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      double para = e[a] * e[b];
      double perp = (a == b ? 1.0 : 0.0) - para;
      D[3 * a + b] = -k * para - kap * perp;
    }
}

// ForceConstants::onsite: D_ii = -sum_{neighbours with ab <= layer} D_ij.
void StiffnessKernel::onsite(int i, int ab, double *D) const {
  for (int a = 0; a < 9; a++) D[a] = 0.0;
  for (const auto &n : surf_.neigh) {
    if (n.i != i || n.ab > ab) continue;
    double t[9];
    offsite(n, t);
    for (int a = 0; a < 9; a++) D[a] -= t[a];
  }
}

// FTStiffnessKernel::pre_compute (src/stiffness_kernels/ft_stiffness.cpp:138-208).
void StiffnessKernel::pre_compute() {
  const int nn = (int)surf_.neigh.size();
  Dij_.assign(9 * (size_t)nn, 0.0);
  for (int n = 0; n < nn; n++) offsite(surf_.neigh[n], &Dij_[9 * (size_t)n]);
  D0ii_.assign(9 * (size_t)surf_.nat, 0.0);
  D1ii_.assign(9 * (size_t)surf_.nat, 0.0);
  for (int i = 0; i < surf_.nat; i++) {
    onsite(i, 0, &D0ii_[9 * (size_t)i]);
    onsite(i, 1, &D1ii_[9 * (size_t)i]);
  }
}

void StiffnessKernel::dynamical_matrices(double qx, double qy, cplx *U0, cplx *U, cplx *V) const {
  const int d = dim_;
  for (int i = 0; i < d * d; i++) U0[i] = U[i] = V[i] = {0.0, 0.0};
  if (kind_ != kFT) {
    // StiffnessKernel::get_dynamical_matrices (src/main/surface_stiffness.cpp:112-270):
    // cell-level U0, U (upper triangle from the per-layer blocks, lower by
    // conjugate transpose) and V (lower triangle), with the phase of the
    // lateral shift between layers
    const int nu = nu_;
    cplx Dl[9 * 25];
    double xc[4], yc[4];
    analytic_layers(qx, qy, Dl, xc, yc);
    auto blk = [&](int r, int c) { return Dl + 9 * (size_t)(r * (nu + 1) + c); };
    auto phase = [&](int i, int j) {
      const double a = (xc[j] - xc[i]) * qx + (yc[j] - yc[i]) * qy;
      return cplx{std::cos(a), std::sin(a)};
    };
    for (int i = 0; i < nu; i++)
      for (int j = i; j < nu; j++) {
        const int r = j - i;
        if (r > nu) continue;
        const cplx *m1 = blk(r, i), *m2 = blk(r, nu);
        const cplx f = i == j ? cplx{1.0, 0.0} : phase(i, j);
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) {
            const cplx p1 = cmul(f, m1[3 * a + b]), p2 = cmul(f, m2[3 * a + b]);
            U0[(3 * i + a) * d + 3 * j + b] = i == j ? m1[3 * a + b] : p1;
            U[(3 * i + a) * d + 3 * j + b] = i == j ? m2[3 * a + b] : p2;
            if (i != j) {
              const cplx q1 = cmul(f, m1[3 * b + a]), q2 = cmul(f, m2[3 * b + a]);
              U0[(3 * j + a) * d + 3 * i + b] = {q1.re, -q1.im};
              U[(3 * j + a) * d + 3 * i + b] = {q2.re, -q2.im};
            }
          }
      }
    for (int i = 0; i < nu; i++)
      for (int j = 0; j <= i; j++) {
        const int r = nu + j - i;
        if (r > nu) continue;
        const cplx *m = blk(r, nu);
        const cplx f = phase(i, j);
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) V[(3 * i + a) * d + 3 * j + b] = cmul(f, m[3 * a + b]);
      }
    return;
  }
  const int nn = (int)surf_.neigh.size();
  for (int n = 0; n < nn; n++) {
    const LatticeNeighbor &nb = surf_.neigh[n];
    if (nb.ab < -1 || nb.ab > 0) continue;  // ab = +1 is the conjugate partner; |ab| > 1 ignored
    double ph = nb.x * qx + nb.y * qy;
    cplx phase = {std::cos(ph), std::sin(ph)};
    const double *Y = &Dij_[9 * (size_t)n];
    cplx *M = nb.ab == 0 ? U : V;
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        size_t idx = (size_t)(3 * nb.i + a) * d + 3 * nb.j + b;
        double y = Y[3 * a + b];
        M[idx].re += phase.re * y;
        M[idx].im += phase.im * y;
        if (nb.ab == 0) {
          U0[idx].re += phase.re * y;
          U0[idx].im += phase.im * y;
        }
      }
  }
  for (int i = 0; i < surf_.nat; i++)
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        size_t idx = (size_t)(3 * i + a) * d + 3 * i + b;
        U0[idx].re += D0ii_[9 * (size_t)i + 3 * a + b];
        U[idx].re += D1ii_[9 * (size_t)i + 3 * a + b];
      }
}

// greens_function_transfer_matrix_stiffness with iterate_Gnn run exactly
// height-1 times (src/main/surface_stiffness.cpp:811-873, 493-548):
//   X = -V U^-1 V^+;  repeat: X = -V (U + X)^-1 V^+;  Phi = U0 + X.
// The recursion X <- -V (U + X)^{-1} V^H on the degrees of freedom V touches.
// X lives on rows(V) x rows(V); (U + X)^{-1} enters through its cols(V) block.
// With S = rows(V) u cols(V) and K the rest, that block is the one of
// (Ut + X)^{-1}, Ut = U_SS - U_SK U_KK^{-1} U_KS the Schur complement of U onto
// S, formed once per wavevector: the recursion then runs on |S| x |S|
// matrices (6 instead of 12 for a four-layer fcc(100) cell).  Returns false
// when S is every degree of freedom or a factorization is not safely
// positive definite (phi then holds scratch); phi receives U0 + X otherwise.
// work holds 6 d^2 entries.
bool StiffnessKernel::reduced_recursion(const cplx *U0, const cplx *U, const cplx *V, cplx *phi,
                                        cplx *work) const {
  const int d = dim_;
  int S[64], K[64], ns = 0, nk = 0;
  for (int i = 0; i < d; i++) {
    bool used = false;
    for (int j = 0; j < d && !used; j++) {
      const cplx a = V[i * d + j], b = V[j * d + i];
      used = a.re != 0.0 || a.im != 0.0 || b.re != 0.0 || b.im != 0.0;
    }
    if (used) S[ns++] = i;
    else K[nk++] = i;
  }
  if (nk == 0 || ns == 0) return false;
  cplx *A = work, *Vs = work + d * d, *X = work + 2 * d * d, *L = work + 3 * d * d, *W = work + 4 * d * d,
       *Y = work + 5 * d * d;
  // Cholesky of U_KK (lower, in L), Y = L^{-1} U_KS, Ut = U_SS - Y^H Y
  for (int j = 0; j < nk; j++) {
    double djj = U[K[j] * d + K[j]].re;
    for (int m = 0; m < j; m++) djj -= L[j * nk + m].re * L[j * nk + m].re + L[j * nk + m].im * L[j * nk + m].im;
    if (!(djj > 1e-12 * std::fabs(U[K[j] * d + K[j]].re))) return false;
    const double ljj = std::sqrt(djj), inv = 1.0 / ljj;
    L[j * nk + j] = {ljj, 0.0};
    for (int i = j + 1; i < nk; i++) {
      double re = U[K[i] * d + K[j]].re, im = U[K[i] * d + K[j]].im;
      for (int m = 0; m < j; m++) {
        const cplx a = L[i * nk + m], b = L[j * nk + m];
        re -= a.re * b.re + a.im * b.im;
        im -= a.im * b.re - a.re * b.im;
      }
      L[i * nk + j] = {re * inv, im * inv};
    }
  }
  for (int i = 0; i < nk; i++) {
    const double inv = 1.0 / L[i * nk + i].re;
    for (int c = 0; c < ns; c++) {
      double re = U[K[i] * d + S[c]].re, im = U[K[i] * d + S[c]].im;
      for (int m = 0; m < i; m++) {
        const cplx a = L[i * nk + m], y = Y[m * ns + c];
        re -= a.re * y.re - a.im * y.im;
        im -= a.re * y.im + a.im * y.re;
      }
      Y[i * ns + c] = {re * inv, im * inv};
    }
  }
  cplx *Ut = phi;  // ns x ns, scratch until the end
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) {
      double re = U[S[a] * d + S[b]].re, im = U[S[a] * d + S[b]].im;
      for (int m = 0; m < nk; m++) {  // - conj(Y[m][a]) Y[m][b]
        const cplx p = Y[m * ns + a], q = Y[m * ns + b];
        re -= p.re * q.re + p.im * q.im;
        im -= p.re * q.im - p.im * q.re;
      }
      Ut[a * ns + b] = {re, im};
    }
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) Vs[a * ns + b] = V[S[a] * d + S[b]];
  // the recursion on S
  bool ok = schur_step_chol(ns, Ut, Vs, X, L, W);
  for (int it = 0; ok && it < height_ - 1; it++) {
    for (int i = 0; i < ns * ns; i++) A[i] = {Ut[i].re + X[i].re, Ut[i].im + X[i].im};
    ok = schur_step_chol(ns, A, Vs, X, L, W);
  }
  if (!ok) return false;
  for (int i = 0; i < d * d; i++) phi[i] = U0[i];
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) {
      phi[S[a] * d + S[b]].re += X[a * ns + b].re;
      phi[S[a] * d + S[b]].im += X[a * ns + b].im;
    }
  return true;
}

bool StiffnessKernel::stiffness(double qx, double qy, cplx *phi, cplx *work) const {
  const int d = dim_, d2 = d * d;
  cplx *U0 = work, *U = work + d2, *V = work + 2 * d2, *Vd = work + 3 * d2, *X = work + 4 * d2,
       *T = work + 5 * d2;
  dynamical_matrices(qx, qy, U0, U, V);
  if (height_ == 0) {
    std::memcpy(phi, U0, sizeof(cplx) * d2);
    return true;
  }
  // Cholesky steps while U + X stays safely positive definite (a Schur
  // complement of the substrate's stiffness matrix); the Gauss-Jordan
  // iteration of the reference otherwise, and at q = 0, where Phi = U0 + X
  // cancels to O(1/height) and the reference's own elimination order keeps
  // the table within 1e-13 of the reference's (Cholesky: 6e-13)
  if (height_ > 0 && !(qx == 0.0 && qy == 0.0) && reduced_recursion(U0, U, V, phi, work + 6 * d2))
    return true;
  if (height_ > 0 && !(qx == 0.0 && qy == 0.0)) {
    cplx *A = Vd, *L = T, *W = phi;  // scratch (Vd is built below if needed)
    bool ok = schur_step_chol(d, U, V, X, L, W);
    for (int it = 0; ok && it < height_ - 1; it++) {
      for (int i = 0; i < d2; i++) A[i] = {U[i].re + X[i].re, U[i].im + X[i].im};
      ok = schur_step_chol(d, A, V, X, L, W);
    }
    if (ok) {
      for (int i = 0; i < d2; i++) phi[i] = {U0[i].re + X[i].re, U0[i].im + X[i].im};
      return true;
    }
  }
  for (int i = 0; i < d; i++)
    for (int j = 0; j < d; j++) Vd[i * d + j] = {-V[j * d + i].re, V[j * d + i].im};
  std::memcpy(X, U, sizeof(cplx) * d2);
  if (!invert(d, X)) return false;
  matmul(d, X, Vd, T);
  matmul(d, V, T, X);
  if (height_ > 0) {
    for (int it = 0; it < height_ - 1; it++) {
      for (int i = 0; i < d2; i++) { X[i].re += U[i].re; X[i].im += U[i].im; }
      if (!invert(d, X)) return false;
      matmul(d, X, Vd, T);
      matmul(d, V, T, X);
    }
  } else {
    // semi-infinite substrate: iterate to a fixed point (eps 1e-8, :836)
    cplx *L = phi;  // scratch until the end
    for (int it = 0; it < 100000; it++) {
      std::memcpy(L, X, sizeof(cplx) * d2);
      for (int i = 0; i < d2; i++) { X[i].re += U[i].re; X[i].im += U[i].im; }
      if (!invert(d, X)) return false;
      matmul(d, X, Vd, T);
      matmul(d, V, T, X);
      double dn = 0.0;
      for (int i = 0; i < d2; i++) {
        double a = X[i].re - L[i].re, b = X[i].im - L[i].im;
        dn += a * a + b * b;
      }
      if (dn <= 1e-16) break;
      if (it == 99999) return false;
    }
  }
  for (int i = 0; i < d2; i++) phi[i] = {U0[i].re + X[i].re, U0[i].im + X[i].im};
  return true;
}

namespace {

// Complex DFT of any length n on the host: recursive mixed-radix decimation
// in time over the prime factors of n, out[k] = sum_t in[t] exp(sign 2 pi i
// t k / n), unscaled.  Cost n * (sum of the prime factors).
class HostDFT {
 public:
  HostDFT(int n, int sign) : n_(n), tw_(n) {
    for (int t = 0; t < n; t++) {
      const double a = 2.0 * kPi * t / n;
      tw_[t] = {std::cos(a), sign * std::sin(a)};
    }
    int m = n;
    for (int p = 2; p * p <= m; p++)
      while (m % p == 0) {
        f_.push_back(p);
        m /= p;
      }
    if (m > 1) f_.push_back(m);
  }
  // in: n entries with the given stride; out: n contiguous entries.
  void run(const cplx *in, int stride, cplx *out) const {
    if (n_ == 1) {
      out[0] = in[0];
      return;
    }
    std::vector<cplx> acc(f_.empty() ? 1 : *std::max_element(f_.begin(), f_.end()));
    rec(in, stride, out, n_, 0, acc.data());
  }

 private:
  int n_;
  std::vector<cplx> tw_;
  std::vector<int> f_;
  // DFT of length n = p * m of in[0], in[stride], ...: p sub-transforms of
  // length m over every p-th input, then the radix-p combination.
  void rec(const cplx *in, int stride, cplx *out, int n, size_t fi, cplx *acc) const {
    if (n == 1) {
      out[0] = in[0];
      return;
    }
    const int p = f_[fi], m = n / p, step = n_ / n;
    for (int r = 0; r < p; r++) rec(in + (size_t)r * stride, stride * p, out + (size_t)r * m, m, fi + 1, acc);
    for (int k = 0; k < m; k++) {
      for (int q = 0; q < p; q++) {
        cplx v = {0.0, 0.0};
        for (int r = 0; r < p; r++) {
          const cplx w = tw_[((size_t)r * (k + (size_t)q * m) % n) * step];
          v = {v.re + out[r * m + k].re * w.re - out[r * m + k].im * w.im,
               v.im + out[r * m + k].re * w.im + out[r * m + k].im * w.re};
        }
        acc[q] = v;
      }
      for (int q = 0; q < p; q++) out[q * m + k] = acc[q];
    }
  }
};

template <class F>
void parallel_for(int n, int nthreads, F f) {
  std::atomic<int> next(0);
  auto worker = [&]() {
    for (int i; (i = next.fetch_add(1)) < n;) f(i);
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(worker);
  worker();
  for (auto &t : th) t.join();
}

// NonperiodicStiffnessKernel::create_and_fill_buffer
// (src/stiffness_kernels/nonperiodic_stiffness.cpp:106-208): the real-space
// Green's function on the minimum-image grid, off-diagonal entries zeroed on
// the far row and column of an even dimension (so the transform stays
// Hermitian), a 2-D transform with exp(+i) per entry, and a 3x3 inverse per
// wavevector.  Only the stored ky columns are transformed along x.
std::string fill_nonperiodic(const StiffnessKernel &k, int nx, int ny, int layout, double *phi,
                             int nthreads) {
  const double xprd = k.box_x() > 0.0 ? k.box_x() : nx, yprd = k.box_y() > 0.0 ? k.box_y() : ny;
  const double dx = xprd / nx, dy = yprd / ny;
  const int nyc = layout == 0 ? ny : ny / 2 + 1;
  const size_t nxy = (size_t)nx * ny;
  std::vector<cplx> g(9 * nxy);  // [entry][ix][iy], transformed along y in place
  const HostDFT fy(ny, +1), fx(nx, +1);
  parallel_for(nx, nthreads, [&](int ix) {
    const int i = ix <= nx / 2 ? ix : ix - nx;
    std::vector<cplx> row(ny), out(ny);
    double G[9];
    std::vector<double> rows(9 * (size_t)ny);
    for (int iy = 0; iy < ny; iy++) {
      const int j = iy <= ny / 2 ? iy : iy - ny;
      k.nonperiodic_green(i, j, dx, dy, G);
      if ((nx % 2 == 0 && ix == nx / 2) || (ny % 2 == 0 && iy == ny / 2))
        G[1] = G[2] = G[3] = G[5] = G[6] = G[7] = 0.0;
      for (int e = 0; e < 9; e++) rows[e * (size_t)ny + iy] = G[e];
    }
    for (int e = 0; e < 9; e++) {
      for (int iy = 0; iy < ny; iy++) row[iy] = {rows[e * (size_t)ny + iy], 0.0};
      fy.run(row.data(), 1, out.data());
      std::memcpy(&g[e * nxy + (size_t)ix * ny], out.data(), sizeof(cplx) * ny);
    }
  });
  std::atomic<int> singular(0), nonherm(0);
  const double inv = 1.0 / ((double)nx * (double)ny);
  parallel_for(nyc, nthreads, [&](int iy) {
    std::vector<cplx> col(9 * (size_t)nx);
    for (int e = 0; e < 9; e++) fx.run(&g[e * nxy + iy], ny, &col[e * (size_t)nx]);
    cplx m[9];
    for (int ix = 0; ix < nx; ix++) {
      for (int e = 0; e < 9; e++) m[e] = col[e * (size_t)nx + ix];
      if (!invert(3, m)) singular.store(1);
      // fill_phi_buffer's Hermitian check (gfmd_misc.cpp:55-76)
      const double tr = m[0].re + m[4].re + m[8].re, tri = m[0].im + m[4].im + m[8].im;
      const double trabs = std::sqrt(tr * tr + tri * tri);
      for (int a = 0; a < 3; a++)
        for (int b = a + 1; b < 3; b++) {
          const double dr = m[3 * a + b].re - m[3 * b + a].re, di = m[3 * a + b].im + m[3 * b + a].im;
          if (std::sqrt(dr * dr + di * di) > 1e-6 * trabs) nonherm.store(1);
        }
      double *o = phi + 2 * ((size_t)ix * nyc + iy) * 9;
      for (int e = 0; e < 9; e++) {
        o[2 * e] = m[e].re * inv;
        o[2 * e + 1] = m[e].im * inv;
      }
    }
  });
  if (singular.load()) return "singular matrix while computing the stiffness kernel";
  if (nonherm.load()) return "kernel is not Hermitian";
  return std::string();
}

}  // namespace

std::string fill_phi_table(const StiffnessKernel &k, int nx, int ny, int layout, double *phi,
                           int nthreads) {
  if (nx < 1 || ny < 1) return "grid dimensions must be positive";
  if (layout != 0 && layout != 1) return "unknown table layout";
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (k.is_nonperiodic()) return fill_nonperiodic(k, nx, ny, layout, phi, nthreads);
  const double xprd = k.box_x() > 0.0 ? k.box_x() : nx, yprd = k.box_y() > 0.0 ? k.box_y() : ny;
  if (k.is_isotropic() && xprd != yprd) return "isotropic kernel works with square surfaces only";
  const int d = k.ndof(), d2 = d * d;
  const int nyc = layout == 0 ? ny : ny / 2 + 1;
  const double inv = 1.0 / ((double)nx * (double)ny);
  std::atomic<int> next(0);
  std::atomic<int> bad_ix(-1), bad_herm(-1);
  auto worker = [&]() {
    std::vector<cplx> work(12 * (size_t)d2), p((size_t)d2);
    for (;;) {
      int ix = next.fetch_add(1);
      if (ix >= nx) break;
      // wavevector folding of fill_phi_buffer (src/main/gfmd_misc.cpp:43-48)
      double qx = (ix <= nx / 2) ? 2.0 * kPi * ix / nx : 2.0 * kPi * (ix - nx) / nx;
      for (int iy = 0; iy < nyc; iy++) {
        double qy = (iy <= ny / 2) ? 2.0 * kPi * iy / ny : 2.0 * kPi * (iy - ny) / ny;
        const bool ok = k.is_isotropic() ? k.isotropic(qx, qy, xprd, yprd, p.data())
                                         : k.stiffness(qx, qy, p.data(), work.data());
        if (!ok) {
          bad_ix.store(ix);
          return;
        }
        // Hermitian check with the reference's tolerance (gfmd_misc.cpp:55-76)
        double tr = 0.0, tri = 0.0;
        for (int i = 0; i < d; i++) { tr += p[i * d + i].re; tri += p[i * d + i].im; }
        double trabs = std::sqrt(tr * tr + tri * tri);
        for (int i = 0; i < d; i++)
          for (int j = 0; j < d; j++) {
            double a = p[i * d + j].re - p[j * d + i].re, b = p[i * d + j].im + p[j * d + i].im;
            if (std::sqrt(a * a + b * b) > 1e-6 * trabs) bad_herm.store(ix);
          }
        double *out = phi + 2 * ((size_t)ix * nyc + iy) * d2;
        for (int e = 0; e < d2; e++) {
          out[2 * e] = p[e].re * inv;
          out[2 * e + 1] = p[e].im * inv;
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; t++) th.emplace_back(worker);
  worker();
  for (auto &t : th) t.join();
  if (bad_ix.load() >= 0) return "singular matrix while computing the stiffness kernel";
  if (bad_herm.load() >= 0) return "kernel is not Hermitian";
  return std::string();
}

}  // namespace gfmd
