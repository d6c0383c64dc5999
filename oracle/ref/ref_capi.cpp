/*
 * ORACLE harness (project code): a C entry point over the reference's own,
 * unmodified sources, compiled where they lie by oracle/ref/Makefile into
 * oracle/_ref/libgfmdref.so.  Used only in the build container, to generate
 * and check the golden fixtures under tests/golden/ and to pin the oracle
 * restatement in oracle/gfmd_oracle.c.
 *
 * The kernel argument string is the stiffness-kernel part of a `fix gfmd`
 * line, e.g. "ft fcc100 1.0 2 pair-potential 1 1.0 height 64"; it is handed
 * to stiffness_kernel_factory the way FixGFMD's constructor does
 * (src/main/fix_gfmd.cpp:195-197).
 */
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "pointers.h"
#include "force.h"
#include "surface_stiffness.h"
#include "gfmd_misc.h"
#include "gfmd_solver_static.h"
#include "table2d.h"

using namespace LAMMPS_NS;

namespace {

thread_local std::string g_last_error;
thread_local double g_box_x = 1.0, g_box_y = 1.0;

struct Env {
  Error error;
  Memory memory{&error};
  Comm comm;
  Domain domain;
  Update update;
  LAMMPS lmp;
  Env() {
    lmp.memory = &memory;
    lmp.error = &error;
    lmp.comm = &comm;
    lmp.domain = &domain;
    lmp.update = &update;
    lmp.screen = nullptr;
    domain.set_cell(g_box_x, g_box_y, 1.0);
  }
};

struct Args {
  std::vector<std::string> tok;
  std::vector<char *> argv;
  explicit Args(const char *s) {
    std::istringstream is(s);
    std::string t;
    while (is >> t) tok.push_back(t);
    for (auto &x : tok) argv.push_back(&x[0]);
    argv.push_back(nullptr);
  }
  int narg() const { return (int)tok.size(); }
};

StiffnessKernel *make_kernel(Env &env, Args &a) {
  if (a.narg() < 1) throw std::runtime_error("empty kernel argument string");
  int carg = 1;
  StiffnessKernel *k = stiffness_kernel_factory(a.argv[0], a.narg(), &carg,
                                                a.argv.data(), &env.domain,
                                                nullptr, &env.memory,
                                                &env.error);
  if (!k) throw std::runtime_error("unknown stiffness kernel '" + a.tok[0] + "'");
  if (carg != a.narg())
    throw std::runtime_error("trailing kernel arguments from '" + a.tok[carg] + "'");
  return k;
}

}  // namespace

extern "C" {

const char *gref_last_error(void) { return g_last_error.c_str(); }

/* Dimension (ndof) and height of a kernel. */
int gref_kernel_info(const char *args, int *ndof, int *height) {
  try {
    Env env;
    Args a(args);
    std::unique_ptr<StiffnessKernel> k(make_kernel(env, a));
    *ndof = k->get_dimension();
    *height = k->get_height();
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

/* Box lengths (LAMMPS' domain->xprd, yprd; the isotropic and nonperiodic
 * kernels read them) of every later call on this thread; default 1 x 1 as
 * the reference's Domain stub. */
int gref_set_box(double xprd, double yprd) {
  g_box_x = xprd;
  g_box_y = yprd;
  return 0;
}

/* Full-grid Phi(q) table exactly as fill_phi_buffer leaves it
 * (src/main/gfmd_misc.cpp:32-101): phi[(ix*ny+iy)*ndof*ndof + i*ndof + j]
 * complex interleaved; linf[ndof/3] from get_force_at_gamma_point. */
int gref_phi_full(const char *args, int nx, int ny, int normalize,
                  double *phi, double *linf) {
  try {
    Env env;
    Args a(args);
    std::unique_ptr<StiffnessKernel> k(make_kernel(env, a));
    int ndof = k->get_dimension();
    int nxy = nx * ny;
    double_complex **buf;
    env.memory.create(buf, nxy, ndof * ndof, "gref:phi");
    fill_phi_buffer(ndof, nx, 0, nx - 1, ny, 0, ny - 1, k.get(), buf,
                    normalize != 0, &env.error);
    std::memcpy(phi, &buf[0][0], sizeof(double_complex) * (size_t)nxy * ndof * ndof);
    env.memory.destroy(buf);
    if (linf) k->get_force_at_gamma_point(linf);
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

/* One call of the reference's GFMDSolverStatic::post_force
 * (src/solvers/gfmd_solver_static.cpp:145-249) on a single process:
 * u, f are [ndof][nx*ny]; returns the energy in *epot and u(q=0) in u0. */
int gref_post_force(const char *args, int nx, int ny, const double *u,
                    double *f, double *epot, double *u0) {
  try {
    Env env;
    Args a(args);
    std::unique_ptr<StiffnessKernel> k(make_kernel(env, a));
    int ndof = k->get_dimension();
    int nxy = nx * ny;
    int carg = 0;
    GFMDSolverStatic solver(&env.lmp, 0, &carg, nullptr);
    solver.set_grid_size(nx, ny, ndof);
    solver.set_kernel(k.get(), true);
    double **ub, **fb;
    env.memory.create(ub, ndof, nxy, "gref:u");
    env.memory.create(fb, ndof, nxy, "gref:f");
    std::memcpy(&ub[0][0], u, sizeof(double) * (size_t)ndof * nxy);
    *epot = solver.post_force(ub, fb, nullptr);
    std::memcpy(f, &fb[0][0], sizeof(double) * (size_t)ndof * nxy);
    if (u0) std::memcpy(u0, solver.get_u0(), sizeof(double) * ndof);
    env.memory.destroy(ub);
    env.memory.destroy(fb);
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

/* One call of the reference's GFMDSolverStatic::prec_gradient
 * (src/solvers/gfmd_solver_static.cpp:253-269): gP from g and Cavg
 * (ndof*ndof), both [ndof][nx*ny]. */
int gref_prec_gradient(const char *args, int nx, int ny, const double *cavg,
                       const double *g, double *gP) {
  try {
    Env env;
    Args a(args);
    std::unique_ptr<StiffnessKernel> k(make_kernel(env, a));
    int ndof = k->get_dimension();
    int nxy = nx * ny;
    int carg = 0;
    GFMDSolverStatic solver(&env.lmp, 0, &carg, nullptr);
    solver.set_grid_size(nx, ny, ndof);
    solver.set_kernel(k.get(), true);
    double **gb, **pb;
    env.memory.create(gb, ndof, nxy, "gref:g");
    env.memory.create(pb, ndof, nxy, "gref:gP");
    std::memcpy(&gb[0][0], g, sizeof(double) * (size_t)ndof * nxy);
    std::vector<double> c(cavg, cavg + (size_t)ndof * ndof);
    solver.prec_gradient(c.data(), gb, pb);
    std::memcpy(gP, &pb[0][0], sizeof(double) * (size_t)ndof * nxy);
    env.memory.destroy(gb);
    env.memory.destroy(pb);
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

/* GFMDSolverFFT::dump_stiffness (greens = 0) or dump_greens_function
 * (greens = 1) of a static solver on an nx x ny grid
 * (src/solvers/gfmd_solver_fft.cpp:294-420); the files go to the current
 * directory. */
int gref_dump(const char *args, int nx, int ny, int greens) {
  try {
    Env env;
    Args a(args);
    std::unique_ptr<StiffnessKernel> k(make_kernel(env, a));
    int carg = 0;
    GFMDSolverStatic solver(&env.lmp, 0, &carg, nullptr);
    solver.set_grid_size(nx, ny, k->get_dimension());
    solver.set_kernel(k.get(), true);
    if (greens) solver.dump_greens_function();
    else solver.dump_stiffness();
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

/* The reference's bicubic map table (Table2D, src/mathutils/table2d.cpp),
 * as FixWallMap builds it (interpolated derivatives, fix_wall_map.cpp:267):
 * values [nx][ny]; at n points (x, y) in pixel units, out[6*i ...] = f, df/dx,
 * df/dy, d2f/dxdx, d2f/dydy, d2f/dxdy. */
int gref_table2d(int nx, int ny, const double *values, int n, const double *x, const double *y,
                 double *out) {
  try {
    Env env;
    double **v;
    env.memory.create(v, nx, ny, "gref:map");
    std::memcpy(&v[0][0], values, sizeof(double) * (size_t)nx * ny);
    {
      Table2D t(nx, ny, v, true, false, &env.error, &env.memory);
      for (int i = 0; i < n; i++) {
        double *o = out + 6 * (size_t)i;
        t.eval(x[i], y[i], o[0], o[1], o[2], o[3], o[4], o[5]);
      }
    }
    env.memory.destroy(v);
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

}  // extern "C"
