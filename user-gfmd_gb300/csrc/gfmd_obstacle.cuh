// Rigid obstacles acting on the atoms of the grid, shared by the solver loops.
//   sphere, exponential wall   e = eps exp(-g/sigma) on the gap g = |r-c| - R
//                              (FixWallMap::eval_exp, src/extras/fix_wall_map.cpp:575-582,
//                              applied to a sphere);
//   sphere, Lennard-Jones 12-6 on the gap, shifted at the cutoff
//                              (FixContactSphere::post_force, src/extras/fix_contact_sphere.cpp:207-264);
//   rigid map, exponential wall on dz = r_z - z_map (normal force only;
//                              FixWallMap::pre_force, src/extras/fix_wall_map.cpp:686-817);
//   rigid map, exponential wall with FixWallMap's bicubic map table evaluated
//                              at the atom's displaced (x, y) and the lateral
//                              force -f_z dz/dx, -f_z dz/dy (fix_wall_map.cpp:686-817,
//                              src/mathutils/table2d.cpp:176-260).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "gfmd_internal.h"

namespace gfmd {

struct Obst {
  int kind;
  double cx, cy, cz, R, eps, sigma, cutoff, offset;
  double c1, c2, c3, c4;  // LJ coefficients
  const double *map;
  int mnx, mny;    // map size (the grid's)
  double map_z0;
  int norm;
  double ax, ay, lx, ly;  // lattice spacing, box
  int nlayer;
  double off[8][3];
  double fz_ext;   // external +z force on each atom of layers l < nlayer
  double gcut;     // effective cutoff on the gap (exp walls without one: 40 sigma)
  double margin;   // extra distance kept in the active-site list
  // FP32 copies for the per-site gating, so sites far from the obstacle cost
  // no FP64 instruction
  float fcx, fcy, fcz, fR, flx, fly, fax, fay, fz0, fnorm;
  float fgate_wall;    // evaluate the wall below this gap estimate
  float fgate_active;  // keep the site in the line-search set below this
  float foff[8][3];
  float feps, finv_sigma, foffset, fgcut;  // map wall in FP32
  const float *mapf;   // FP32 copy of the map (may be NULL: then map is read)
  // FP32 sphere walls and gating (sphere_off): the centre's nearest site
  // (icx, icy) in [0, nx) x [0, ny), per layer the residual offsets
  // (icx ax + off_x - cx, icy ay + off_y - cy) and off_z - cz + R
  int icx, icy;
  float fres[8][3];
  float fc1, fc2, fc3, fc4;  // LJ coefficients in FP32
  // gates of the CG kernels on cg_gate's value: evaluate the wall below gw,
  // keep the site in the line-search set below ga (spheres: G (2R + G) for
  // the gap ranges G, as |d|^2 - R^2 < G (2R + G) <=> gap < G; maps: gaps)
  float gw, ga;
};

// Exponential map wall in FP32 on atom height rz at site s: energy and z force.
__device__ __forceinline__ void map_wall_f(const Obst &o, size_t s, float rz, float &e, float &fz) {
  const float zm = (o.mapf ? o.mapf[s] : (float)o.map[s]) + o.fz0;
  const float dz = o.fnorm * (rz - zm);
  if (dz >= o.fgcut) {
    e = 0.0f;
    fz = 0.0f;
    return;
  }
  const float ex = o.feps * expf(-dz * o.finv_sigma);
  e = ex - o.foffset;
  fz = o.fnorm * ex * o.finv_sigma;
}

// Offset of the atom of layer l at site (ix, iy), displaced by (ux, uy, uz),
// from a sphere's centre, in FP32: dx, dy, the height w above the sphere's
// lowest point and s = |d|^2 - R^2 = dx^2 + dy^2 + w (w - 2R).  The lateral
// offsets start from the integer distance to the centre's nearest site
// (minimum image in integers), so their rounding is relative to the offset
// itself and not to the box; s has no cancellation against R^2, so the gap
// s / (|d| + R) keeps FP32 precision relative to the gap.
struct SphereOff {
  float dx, dy, w, s;
};
__device__ __forceinline__ SphereOff sphere_off(const Obst &o, int nx, int ny, int ix, int iy, int l, float ux,
                                                float uy, float uz) {
  int jx = ix - o.icx, jy = iy - o.icy;
  if (2 * jx >= nx) jx -= nx;
  else if (2 * jx < -nx) jx += nx;
  if (2 * jy >= ny) jy -= ny;
  else if (2 * jy < -ny) jy += ny;
  SphereOff q;
  q.dx = fmaf((float)jx, o.fax, o.fres[l][0]) + ux;
  q.dy = fmaf((float)jy, o.fay, o.fres[l][1]) + uy;
  q.w = o.fres[l][2] + uz;
  q.s = fmaf(q.dx, q.dx, fmaf(q.dy, q.dy, q.w * (q.w - 2.0f * o.fR)));
  return q;
}

// Sphere wall (exponential or Lennard-Jones on the gap) in FP32 at offset q:
// energy, force and the curvature dir^T H dir; false beyond the range.
__device__ __forceinline__ bool sphere_wall_f(const Obst &o, const SphereOff &q, const float dir[3], float &e,
                                              float f[3], float &curv) {
  const float dz = q.w - o.fR;
  const float rho2 = fmaf(q.dx, q.dx, fmaf(q.dy, q.dy, dz * dz));
  const float ir = rsqrtf(rho2);
  const float g = q.s / fmaf(rho2, ir, o.fR);
  if (!(g < o.fgcut)) return false;
  float F, E2;  // F = -dE/dg, E2 = d2E/dg2
  if (o.kind == GFMD_OBST_SPHERE_EXP) {
    const float ex = o.feps * expf(-g * o.finv_sigma);
    e = ex - o.foffset;
    F = ex * o.finv_sigma;
    E2 = F * o.finv_sigma;
  } else {
    const float gi = 1.0f / g, g2 = gi * gi, g6 = g2 * g2 * g2;
    e = g6 * (o.fc3 * g6 - o.fc4) - o.foffset;
    F = g6 * (o.fc1 * g6 - o.fc2) * gi;
    E2 = g6 * g2 * (13.0f * o.fc1 * g6 - 7.0f * o.fc2);
  }
  const float n0 = q.dx * ir, n1 = q.dy * ir, n2 = dz * ir;
  f[0] = F * n0;
  f[1] = F * n1;
  f[2] = F * n2;
  const float dn = dir[0] * n0 + dir[1] * n1 + dir[2] * n2;
  const float dd = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
  // Hessian of E(|r-c|): E'' n n^T + (E'/rho)(1 - n n^T), E' = -F
  curv = E2 * dn * dn - F * ir * (dd - dn * dn);
  return true;
}

// FixWallMap's bicubic map table (Table2D with interpolated derivatives,
// src/mathutils/table2d.cpp): on the periodic pixel cell [i, i+1] x [j, j+1]
// the bicubic with the corner values, central-difference slopes
// (z[i+1] - z[i-1]) / 2 along each axis and zero cross derivatives, written in
// the cubic Hermite basis.  (x, y) in pixel units; outputs z and its first and
// second derivatives in pixel units.
struct MapBicubic {
  double z, zx, zy, zxx, zyy, zxy;
};
template <typename T>
__device__ __forceinline__ T map_at(const T *m, int nx, int ny, int i, int j) {
  i %= nx;
  if (i < 0) i += nx;
  j %= ny;
  if (j < 0) j += ny;
  return m[(size_t)i * ny + j];
}
__device__ __forceinline__ MapBicubic map_bicubic(const double *m, int nx, int ny, double x, double y) {
  const double fx = floor(x), fy = floor(y);
  const int i0 = (int)fx, j0 = (int)fy;
  const double t = x - fx, u = y - fy;
  // Hermite basis H0, H1 (values at 0, 1), G0, G1 (slopes at 0, 1) and derivatives
  const double t2 = t * t, t3 = t2 * t, u2 = u * u, u3 = u2 * u;
  const double hx[4] = {2 * t3 - 3 * t2 + 1, -2 * t3 + 3 * t2, t3 - 2 * t2 + t, t3 - t2};
  const double dx1[4] = {6 * t2 - 6 * t, -6 * t2 + 6 * t, 3 * t2 - 4 * t + 1, 3 * t2 - 2 * t};
  const double dx2[4] = {12 * t - 6, -12 * t + 6, 6 * t - 4, 6 * t - 2};
  const double hy[4] = {2 * u3 - 3 * u2 + 1, -2 * u3 + 3 * u2, u3 - 2 * u2 + u, u3 - u2};
  const double dy1[4] = {6 * u2 - 6 * u, -6 * u2 + 6 * u, 3 * u2 - 4 * u + 1, 3 * u2 - 2 * u};
  const double dy2[4] = {12 * u - 6, -12 * u + 6, 6 * u - 4, 6 * u - 2};
  MapBicubic r{0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const double f = map_at(m, nx, ny, i0 + a, j0 + b);
      const double fxs = 0.5 * (map_at(m, nx, ny, i0 + a + 1, j0 + b) - map_at(m, nx, ny, i0 + a - 1, j0 + b));
      const double fys = 0.5 * (map_at(m, nx, ny, i0 + a, j0 + b + 1) - map_at(m, nx, ny, i0 + a, j0 + b - 1));
      // value term H_a(t) H_b(u), slope terms G_a(t) H_b(u) and H_a(t) G_b(u)
      r.z += f * hx[a] * hy[b] + fxs * hx[2 + a] * hy[b] + fys * hx[a] * hy[2 + b];
      r.zx += f * dx1[a] * hy[b] + fxs * dx1[2 + a] * hy[b] + fys * dx1[a] * hy[2 + b];
      r.zy += f * hx[a] * dy1[b] + fxs * hx[2 + a] * dy1[b] + fys * hx[a] * dy1[2 + b];
      r.zxx += f * dx2[a] * hy[b] + fxs * dx2[2 + a] * hy[b] + fys * dx2[a] * hy[2 + b];
      r.zyy += f * hx[a] * dy2[b] + fxs * hx[2 + a] * dy2[b] + fys * hx[a] * dy2[2 + b];
      r.zxy += f * dx1[a] * dy1[b] + fxs * dx1[2 + a] * dy1[b] + fys * dx1[a] * dy1[2 + b];
    }
  return r;
}
struct WallOut {
  double e;        // energy
  double f[3];     // force on the atom
  double curv;     // h^T (d2E/dr2) h for the given direction
};

// Obstacle energy, force and curvature along dir at position r.  The
// bicubic map wall is compiled in only with BIC = true: its code would raise
// the register count of every kernel that evaluates walls, so only the
// kernels of the paths that offer it (CG, gfmd_obstacle_force) carry it.
template <bool BIC = false>
__device__ __forceinline__ WallOut wall_eval(const Obst &o, int s_ix, int s_iy, size_t site,
                                             const double r[3], const double dir[3]) {
  WallOut w{0.0, {0.0, 0.0, 0.0}, 0.0};
  if (o.kind == GFMD_OBST_SPHERE_EXP || o.kind == GFMD_OBST_SPHERE_LJ) {
    double d[3] = {r[0] - o.cx, r[1] - o.cy, r[2] - o.cz};
    // minimum image in x and y (periodic grid)
    d[0] -= o.lx * rint(d[0] / o.lx);
    d[1] -= o.ly * rint(d[1] / o.ly);
    const double rho = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double g = rho - o.R;
    if (g >= o.gcut) return w;
    double e, F, E2;  // E(g), F = -dE/dg, d2E/dg2
    if (o.kind == GFMD_OBST_SPHERE_EXP) {
      const double ex = o.eps * exp(-g / o.sigma);
      e = ex - o.offset;
      F = ex / o.sigma;
      E2 = F / o.sigma;
    } else {
      const double ginv = 1.0 / g, g2 = ginv * ginv, g6 = g2 * g2 * g2;
      e = g6 * (o.c3 * g6 - o.c4) - o.offset;
      F = g6 * (o.c1 * g6 - o.c2) * ginv;
      E2 = g6 * g2 * (13.0 * o.c1 * g6 - 7.0 * o.c2);
    }
    const double ir = 1.0 / rho;
    const double n[3] = {d[0] * ir, d[1] * ir, d[2] * ir};
    w.e = e;
    w.f[0] = F * n[0];
    w.f[1] = F * n[1];
    w.f[2] = F * n[2];
    const double dn = dir[0] * n[0] + dir[1] * n[1] + dir[2] * n[2];
    const double dd = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
    // Hessian of E(|r-c|): E'' n n^T + (E'/rho)(1 - n n^T), E' = -F
    w.curv = E2 * dn * dn - F * ir * (dd - dn * dn);
  } else if (o.kind == GFMD_OBST_MAP_EXP) {
    const double zm = o.map[site] + o.map_z0;
    const double dz = o.norm * (r[2] - zm);
    if (dz >= o.gcut) return w;
    const double ex = o.eps * exp(-dz / o.sigma);
    w.e = ex - o.offset;
    w.f[2] = o.norm * ex / o.sigma;
    w.curv = ex / (o.sigma * o.sigma) * dir[2] * dir[2];
  } else if (BIC && o.kind == GFMD_OBST_MAP_BICUBIC) {
    // map pixel (i, j) sits at (i ax, j ay): evaluate at the displaced position
    const MapBicubic mb = map_bicubic(o.map, o.mnx, o.mny, r[0] / o.ax, r[1] / o.ay);
    const double zx = mb.zx / o.ax, zy = mb.zy / o.ay;
    const double zxx = mb.zxx / (o.ax * o.ax), zyy = mb.zyy / (o.ay * o.ay), zxy = mb.zxy / (o.ax * o.ay);
    const double dz = o.norm * (r[2] - (mb.z + o.map_z0));
    if (dz >= o.gcut) return w;
    const double ex = o.eps * exp(-dz / o.sigma);
    const double fz = o.norm * ex / o.sigma;
    w.e = ex - o.offset;
    w.f[0] = -fz * zx;
    w.f[1] = -fz * zy;
    w.f[2] = fz;
    // E = eps exp(-dz/sigma), grad dz = norm (-zx, -zy, 1):
    // d^T H d = E/sigma^2 (grad dz . d)^2 + E/sigma norm (zxx dx^2 + 2 zxy dx dy + zyy dy^2)
    const double gd = o.norm * (dir[2] - zx * dir[0] - zy * dir[1]);
    w.curv = ex / (o.sigma * o.sigma) * gd * gd +
             ex / o.sigma * o.norm * (zxx * dir[0] * dir[0] + 2.0 * zxy * dir[0] * dir[1] + zyy * dir[1] * dir[1]);
  }
  return w;
}

// Cheap FP32 estimate of the gap of an atom (no minimum image subtleties
// beyond what the margin covers); used to skip the FP64 evaluation far away.
__device__ __forceinline__ float gap_estimate(const Obst &o, size_t site, const double r[3]) {
  if (o.kind == GFMD_OBST_MAP_EXP) {
    return (float)o.norm * ((float)r[2] - (float)(o.map[site] + o.map_z0));
  }
  if (o.kind == GFMD_OBST_MAP_BICUBIC) return -1e30f;  // no gating: every site is evaluated
  float dx = (float)(r[0] - o.cx), dy = (float)(r[1] - o.cy), dz = (float)(r[2] - o.cz);
  const float lx = (float)o.lx, ly = (float)o.ly;
  dx -= lx * rintf(dx / lx);
  dy -= ly * rintf(dy / ly);
  return sqrtf(dx * dx + dy * dy + dz * dz) - (float)o.R;
}

// FP32 gap estimate from an FP32 position (gating only).
__device__ __forceinline__ float gap_estimate_f(const Obst &o, size_t site, const float r[3]) {
  if (o.kind == GFMD_OBST_MAP_EXP) {
    const float zm = o.mapf ? o.mapf[site] : (float)o.map[site];
    return o.fnorm * (r[2] - (zm + o.fz0));
  }
  if (o.kind == GFMD_OBST_MAP_BICUBIC) return -1e30f;  // no gating: every site is evaluated
  float dx = r[0] - o.fcx, dy = r[1] - o.fcy, dz = r[2] - o.fcz;
  dx -= o.flx * rintf(dx / o.flx);
  dy -= o.fly * rintf(dy / o.fly);
  return sqrtf(dx * dx + dy * dy + dz * dz) - o.fR;
}

inline Obst make_obst(const gfmd_obstacle_t *ob, const Geom &g) {
  Obst o{};
  o.kind = ob ? ob->kind : GFMD_OBST_NONE;
  if (!ob) return o;
  o.cx = ob->center[0];
  o.cy = ob->center[1];
  o.cz = ob->center[2];
  o.R = ob->radius;
  o.eps = ob->epsilon;
  o.sigma = ob->sigma;
  o.cutoff = ob->cutoff;
  o.map = ob->d_map;
  o.mnx = g.nx;
  o.mny = g.ny;
  o.map_z0 = ob->map_z0;
  o.norm = ob->norm == 0 ? 1 : ob->norm;
  o.fz_ext = ob->fz_ext;
  o.ax = ob->lattice[0] > 0 ? ob->lattice[0] : 1.0;
  o.ay = ob->lattice[1] > 0 ? ob->lattice[1] : 1.0;
  o.lx = o.ax * g.nx;
  o.ly = o.ay * g.ny;
  o.nlayer = std::min(g.ndof / 3, ob->nlayer > 0 ? ob->nlayer : g.ndof / 3);
  for (int l = 0; l < 8; l++)
    for (int c = 0; c < 3; c++) o.off[l][c] = ob->layer_offset[l][c];
  if (o.kind == GFMD_OBST_SPHERE_LJ) {
    o.c1 = 48.0 * o.eps * std::pow(o.sigma, 12.0);
    o.c2 = 24.0 * o.eps * std::pow(o.sigma, 6.0);
    o.c3 = 4.0 * o.eps * std::pow(o.sigma, 12.0);
    o.c4 = 4.0 * o.eps * std::pow(o.sigma, 6.0);
    if (o.cutoff > 0.0) {
      const double r2 = 1.0 / (o.cutoff * o.cutoff), r6 = r2 * r2 * r2;
      o.offset = r6 * (o.c3 * r6 - o.c4);
    }
  } else if (o.cutoff > 0.0) {
    o.offset = o.eps * std::exp(-o.cutoff / o.sigma);
  }
  // exponential walls without a cutoff: beyond 40 sigma the force is below
  // 4e-18 eps/sigma, far under any force tolerance
  o.gcut = o.cutoff > 0.0 ? o.cutoff : (o.kind == GFMD_OBST_SPHERE_LJ ? 1e30 : 40.0 * o.sigma);
  o.margin = 10.0 * o.sigma + 1.0;
  o.fcx = (float)o.cx;
  o.fcy = (float)o.cy;
  o.fcz = (float)o.cz;
  o.fR = (float)o.R;
  o.flx = (float)o.lx;
  o.fly = (float)o.ly;
  o.fax = (float)o.ax;
  o.fay = (float)o.ay;
  o.fz0 = (float)o.map_z0;
  o.fnorm = (float)o.norm;
  o.fgate_wall = (float)o.gcut + 0.01f * (float)o.gcut + 1e-3f;
  o.fgate_active = (float)(o.gcut + o.margin);
  for (int l = 0; l < 8; l++)
    for (int c = 0; c < 3; c++) o.foff[l][c] = (float)o.off[l][c];
  if (o.kind == GFMD_OBST_SPHERE_EXP || o.kind == GFMD_OBST_SPHERE_LJ) {
    const double kx = std::nearbyint(o.cx / o.ax), ky = std::nearbyint(o.cy / o.ay);
    o.icx = (int)(((long long)kx % g.nx + g.nx) % g.nx);
    o.icy = (int)(((long long)ky % g.ny + g.ny) % g.ny);
    for (int l = 0; l < 8; l++) {
      o.fres[l][0] = (float)(kx * o.ax + o.off[l][0] - o.cx);
      o.fres[l][1] = (float)(ky * o.ay + o.off[l][1] - o.cy);
      o.fres[l][2] = (float)(o.off[l][2] - o.cz + o.R);
    }
    const double gw = o.fgate_wall, ga = o.fgate_active;
    o.gw = (float)(gw * (2.0 * o.R + gw));
    o.ga = (float)(ga * (2.0 * o.R + ga));
  } else {
    o.gw = o.fgate_wall;
    o.ga = o.fgate_active;
  }
  o.fc1 = (float)o.c1;
  o.fc2 = (float)o.c2;
  o.fc3 = (float)o.c3;
  o.fc4 = (float)o.c4;
  o.mapf = nullptr;
  o.feps = (float)o.eps;
  o.finv_sigma = o.sigma > 0.0 ? (float)(1.0 / o.sigma) : 0.0f;
  o.foffset = (float)o.offset;
  o.fgcut = (float)o.gcut;
  return o;
}

// Total force F_el(u) + F_w(u) of FP64 displacements with handle hh on
// stream st: energy, max |f_i| and |f|^2 (synchronizes st).
cudaError_t report_total_force(gfmd_solver *hh, cudaStream_t st, const Obst &o, const double *u,
                               double *E, double *fmax, double *f2);

}  // namespace gfmd
