// Host-side Phi(q) table producer for the `ft` stiffness-kernel style with the
// `pair-potential` force-constant model on the sc100, fcc100 and fcc111
// crystal surfaces, for the analytic `sc100` and `fcc100` styles, and for the
// continuum `isotropic` and `nonperiodic` styles.
//
// Reference behaviour restated (USER-GFMD):
//   surfaces             src/surfaces/{sc100,fcc100,fcc111}_surface.cpp,
//                        CrystalSurface::supercell / reverse_indices /
//                        set_cell_and_scale_atoms / compute_neighbor_list /
//                        identify_neighbor_shells
//                        (src/main/crystal_surface.cpp:166-330, 428-548)
//   force constants      FCPairPotential (src/force_constants/fc_pair_potential.cpp:32-181),
//                        ForceConstants::onsite (src/main/force_constants.cpp:63-83)
//   dynamical matrices   FTStiffnessKernel::get_dynamical_matrices
//                        (src/stiffness_kernels/ft_stiffness.cpp:216-305)
//   transfer matrix      greens_function_transfer_matrix_stiffness + iterate_Gnn
//                        (src/main/surface_stiffness.cpp:493-548, 811-873)
//   table fill           fill_phi_buffer (src/main/gfmd_misc.cpp:32-101)
//   analytic styles      SC100StiffnessKernel (src/stiffness_kernels/sc100_stiffness.cpp:137-227),
//                        FCC100StiffnessKernel (src/stiffness_kernels/fcc100_stiffness.cpp:57-487),
//                        cell matrices from per-layer blocks in
//                        StiffnessKernel::get_dynamical_matrices
//                        (src/main/surface_stiffness.cpp:112-270)
//   continuum styles     IsotropicStiffnessKernel (src/stiffness_kernels/isotropic_stiffness.cpp:43-146),
//                        NonperiodicStiffnessKernel (src/stiffness_kernels/nonperiodic_stiffness.cpp:44-242)
//
// It exists so that a machine without the reference tree can still build the
// tables the force path needs; inside LAMMPS the reference's own
// fill_phi_buffer produces them and hands them to gfmd_set_phi.
#ifndef GFMD_GB300_STIFFNESS_H
#define GFMD_GB300_STIFFNESS_H

#include <string>
#include <vector>

namespace gfmd {

struct cplx {
  double re, im;
};

struct LatticeNeighbor {
  int i, j;       // root atom, neighbour atom (indices within the surface cell)
  int x, y, ab;   // cell offset of the neighbour (ab: layers, +1 = above)
  double r[3];    // r_i - r_j - cell.(x,y,ab)
  double rnorm;
  int shell;      // neighbour shell, 0 = nearest
};

struct CrystalSurface {
  std::string name;
  double cell[9];              // row-major, lattice vectors are the columns
  double invcell[9];
  int nat = 0;
  std::vector<double> pos;     // 3*nat
  std::vector<LatticeNeighbor> neigh;

  void set_cell(const double *c);
  void supercell_z(int nz);
  void reverse_indices();
  void scale_cell(double a);
  void compute_neighbor_list(double rcut);
};

class StiffnessKernel {
 public:
  // Parses the stiffness-kernel part of a `fix gfmd` line starting at
  // tok[pos] (the keyword) and advances pos past what it consumed.
  // Throws std::runtime_error with a message on malformed input.
  static StiffnessKernel *create(const std::vector<std::string> &tok, size_t &pos);
  static StiffnessKernel *create_analytic(const std::string &kw, const std::vector<std::string> &tok,
                                          size_t &pos);
  static StiffnessKernel *create_continuum(const std::string &kw, const std::vector<std::string> &tok,
                                           size_t &pos);

  // Lateral box lengths (LAMMPS domain->xprd, yprd), read by the isotropic
  // and nonperiodic styles.  Zero (the default) means one lattice spacing per
  // grid point: xprd = nx, yprd = ny of the table being filled.
  void set_box(double xprd, double yprd) { box_x_ = xprd; box_y_ = yprd; }
  double box_x() const { return box_x_; }
  double box_y() const { return box_y_; }
  bool is_isotropic() const { return kind_ == kIsotropic; }
  bool is_nonperiodic() const { return kind_ == kNonperiodic; }
  // Isotropic elastic half-space at one wavevector (3x3); false if singular.
  bool isotropic(double qx, double qy, double xprd, double yprd, cplx *phi) const;
  // Real-space surface Green's function of the nonperiodic style at grid
  // offset (i, j) with spacing (dx, dy): G[3*a + b] = displacement a under
  // unit force b spread uniformly over one dx x dy cell.
  void nonperiodic_green(int i, int j, double dx, double dy, double *G) const;

  int ndof() const { return dim_; }
  int height() const { return height_; }
  // Linear force per layer at the gamma point.  For `pair-potential` this is
  // zero even when the `linf` keyword is given: the reference parses and
  // checks the values but FCPairPotential::linear
  // (src/force_constants/fc_pair_potential.cpp:184-191) does not override
  // ForceConstants::linear (src/main/force_constants.cpp:88-94), so
  // FTStiffnessKernel::get_force_at_gamma_point returns zeros.
  // The analytic fcc100 style returns its `linf` values
  // (FCC100StiffnessKernel::get_force_at_gamma_point, fcc100_stiffness.cpp:482-487).
  std::vector<double> linf() const {
    if (kind_ == kFCC100) return linf_;
    return std::vector<double>(kind_ == kFT ? surf_.nat : nu_, 0.0);
  }
  // The values given with the `linf` keyword.
  const std::vector<double> &linf_keyword() const { return linf_; }
  const std::string &name() const { return name_; }
  // The crystal surface of an `ft` kernel (cell, basis, neighbour list).
  const CrystalSurface &surface() const { return surf_; }

  // U0, U, V at one wavevector (each dim*dim, row-major).
  void dynamical_matrices(double qx, double qy, cplx *U0, cplx *U, cplx *V) const;
  // Phi(q) = U0 + V T_N (zero-force transfer matrix over `height` layers);
  // work holds at least 12*dim*dim entries.  Returns false if a matrix was
  // singular.
  bool stiffness(double qx, double qy, cplx *phi, cplx *work) const;
  bool reduced_recursion(const cplx *U0, const cplx *U, const cplx *V, cplx *phi, cplx *work) const;

 private:
  // `ft` (force constants on a crystal surface), the analytic lattice styles,
  // or the continuum styles
  enum Kind { kFT, kSC100, kFCC100, kIsotropic, kNonperiodic };
  Kind kind_ = kFT;
  double poisson_ = 0.0, shear_ = 1.0, gamma_ = 1.0;  // isotropic / nonperiodic
  double box_x_ = 0.0, box_y_ = 0.0;
  int nu_ = 1;      // layers of the analytic styles
  int z_ = 1;       // surface normal of the analytic fcc100 style
  std::string name_;
  CrystalSurface surf_;
  int dim_ = 3;
  int height_ = 0;
  double k_[3] = {0, 0, 0}, kappa_[3] = {0, 0, 0};
  std::vector<double> linf_;
  std::vector<double> D0ii_, D1ii_, Dij_;  // on-site (per atom) and off-site (per neighbour)

  // Per-layer blocks of the analytic styles in (nu+1)^2 slots of 9 entries
  // (row 0: U0..U_{nu-1}, U; row 1: V0.., V; row 2: W0.., W) and the lateral
  // shift of every layer in cell units.
  void analytic_layers(double qx, double qy, cplx *D, double *xc, double *yc) const;
  void offsite(const LatticeNeighbor &n, double *D) const;
  void onsite(int i, int ab, double *D) const;
  void pre_compute();
};

// Fills the Phi table for an nx*ny grid, scaled by 1/(nx*ny).
//   layout 0 (full):  phi[(ix*ny+iy)*dim*dim + i*dim + j], every grid point,
//                     identical in meaning to fill_phi_buffer's output;
//   layout 1 (half):  phi[(ix*(ny/2+1)+ky)*dim*dim + ...], ky = 0..ny/2.
// Runs on `nthreads` host threads (<= 0: all).  Returns an empty string on
// success, else an error message.
std::string fill_phi_table(const StiffnessKernel &k, int nx, int ny, int layout,
                           double *phi, int nthreads);

}  // namespace gfmd

#endif
