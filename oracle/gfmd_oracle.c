/*
 * ORACLE — test infrastructure, not product code.  See gfmd_oracle.h.
 *
 * The FFT here stands in for LAMMPS' FFT3d (KSPACE fft3d_wrap.h over FFTW3
 * or KISS FFT), which the reference calls from
 * src/solvers/gfmd_solver_fft.cpp:116 (forward) and :181 (backward) and which
 * is not part of the reference tree.  It is a textbook mixed-radix Stockham
 * transform (radix 4, 2, 3, 5 and a direct DFT for any other prime factor),
 * unscaled in both directions like FFT3d with scaled = 0.
 */
#include "gfmd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_STAGES 64
#define ORC_PI 3.14159265358979323846264338327950288

struct orc_fft_plan {
    int n;
    int nstages;
    int radix[ORC_MAX_STAGES];
    int span[ORC_MAX_STAGES];      /* product of the radices before stage s */
    double *tw[ORC_MAX_STAGES];    /* span*radix forward twiddles, [k][r] */
    double *roots[ORC_MAX_STAGES]; /* radix forward roots exp(-2 pi i m/R) */
};

static void orc_factor(int n, int *radix, int *nst)
{
    int k = 0;
    while (n % 4 == 0) { radix[k++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[k++] = 2; n /= 2; }
    for (int p = 3; n > 1; p += 2) {
        while (n % p == 0) { radix[k++] = p; n /= p; }
    }
    *nst = k;
}

orc_fft_plan *orc_fft_plan_create(int n)
{
    if (n < 1) return NULL;
    orc_fft_plan *p = (orc_fft_plan *)calloc(1, sizeof(orc_fft_plan));
    p->n = n;
    orc_factor(n, p->radix, &p->nstages);
    int span = 1;
    for (int s = 0; s < p->nstages; s++) {
        int R = p->radix[s];
        int L = span * R;
        p->span[s] = span;
        p->tw[s] = (double *)malloc(sizeof(double) * 2 * (size_t)L);
        for (int k = 0; k < span; k++) {
            for (int r = 0; r < R; r++) {
                /* exp(-2 pi i r k / L), argument reduced exactly */
                long m = ((long)r * k) % L;
                double a = -2.0 * ORC_PI * (double)m / (double)L;
                p->tw[s][2 * (k * R + r)] = cos(a);
                p->tw[s][2 * (k * R + r) + 1] = sin(a);
            }
        }
        p->roots[s] = (double *)malloc(sizeof(double) * 2 * (size_t)R);
        for (int m = 0; m < R; m++) {
            double a = -2.0 * ORC_PI * (double)m / (double)R;
            p->roots[s][2 * m] = cos(a);
            p->roots[s][2 * m + 1] = sin(a);
        }
        span = L;
    }
    return p;
}

void orc_fft_plan_destroy(orc_fft_plan *p)
{
    if (!p) return;
    for (int s = 0; s < p->nstages; s++) {
        free(p->tw[s]);
        free(p->roots[s]);
    }
    free(p);
}

/* One Stockham stage: in[j + r*n/R] -> out[(j/Ns)*Ns*R + j%Ns + r*Ns]. */
static void orc_stage(const orc_fft_plan *p, int s, const double *in,
                      double *out, int sign)
{
    const int n = p->n, R = p->radix[s], Ns = p->span[s], m = n / R;
    const double *tw = p->tw[s];
    const double *roots = p->roots[s];
    const double sg = (double)sign * -1.0; /* +1 for forward tables as is */
    double vr[64], vi[64];
    double *gr = NULL, *gi = NULL;
    if (R > 64) {
        gr = (double *)malloc(sizeof(double) * 2 * (size_t)R);
        gi = gr + R;
    }
    double *xr = R > 64 ? gr : vr, *xi = R > 64 ? gi : vi;

    for (int j = 0; j < m; j++) {
        int k = j % Ns;
        for (int r = 0; r < R; r++) {
            double ar = in[2 * (j + r * m)], ai = in[2 * (j + r * m) + 1];
            double wr = tw[2 * (k * R + r)], wi = sg * tw[2 * (k * R + r) + 1];
            xr[r] = ar * wr - ai * wi;
            xi[r] = ar * wi + ai * wr;
        }
        int base = (j / Ns) * Ns * R + k;
        if (R == 2) {
            out[2 * base] = xr[0] + xr[1];
            out[2 * base + 1] = xi[0] + xi[1];
            out[2 * (base + Ns)] = xr[0] - xr[1];
            out[2 * (base + Ns) + 1] = xi[0] - xi[1];
        } else if (R == 4) {
            double s0r = xr[0] + xr[2], s0i = xi[0] + xi[2];
            double d0r = xr[0] - xr[2], d0i = xi[0] - xi[2];
            double s1r = xr[1] + xr[3], s1i = xi[1] + xi[3];
            double d1r = xr[1] - xr[3], d1i = xi[1] - xi[3];
            /* multiply d1 by i^sign: sign=-1 -> -i */
            double er = (double)(-sign) * d1i, ei = (double)sign * d1r;
            out[2 * base] = s0r + s1r;
            out[2 * base + 1] = s0i + s1i;
            out[2 * (base + Ns)] = d0r + er;
            out[2 * (base + Ns) + 1] = d0i + ei;
            out[2 * (base + 2 * Ns)] = s0r - s1r;
            out[2 * (base + 2 * Ns) + 1] = s0i - s1i;
            out[2 * (base + 3 * Ns)] = d0r - er;
            out[2 * (base + 3 * Ns) + 1] = d0i - ei;
        } else {
            for (int t = 0; t < R; t++) {
                double sr = 0.0, si = 0.0;
                for (int q = 0; q < R; q++) {
                    int e = (int)(((long)q * t) % R);
                    double wr = roots[2 * e], wi = sg * roots[2 * e + 1];
                    sr += xr[q] * wr - xi[q] * wi;
                    si += xr[q] * wi + xi[q] * wr;
                }
                out[2 * (base + t * Ns)] = sr;
                out[2 * (base + t * Ns) + 1] = si;
            }
        }
    }
    free(gr);
}

void orc_fft_exec(const orc_fft_plan *p, double *data, double *work, int sign)
{
    double *a = data, *b = work;
    for (int s = 0; s < p->nstages; s++) {
        orc_stage(p, s, a, b, sign);
        double *t = a; a = b; b = t;
    }
    if (a != data) memcpy(data, a, sizeof(double) * 2 * (size_t)p->n);
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_fft2d(double *data, int nx, int ny, int flag, int nthreads)
{
    if (nx < 1 || ny < 1 || (flag != 1 && flag != -1)) return -1;
    int sign = flag == 1 ? -1 : +1;
    if (nthreads <= 0) nthreads = orc_max_threads();
    orc_fft_plan *py = orc_fft_plan_create(ny);
    orc_fft_plan *px = orc_fft_plan_create(nx);
    /* rows along y (contiguous) */
#pragma omp parallel num_threads(nthreads)
    {
        double *work = (double *)malloc(sizeof(double) * 2 * (size_t)(nx > ny ? nx : ny));
        double *col = (double *)malloc(sizeof(double) * 2 * (size_t)nx);
#pragma omp for schedule(static)
        for (int ix = 0; ix < nx; ix++)
            orc_fft_exec(py, data + 2 * (size_t)ix * ny, work, sign);
#pragma omp for schedule(static)
        for (int iy = 0; iy < ny; iy++) {
            for (int ix = 0; ix < nx; ix++) {
                col[2 * ix] = data[2 * ((size_t)ix * ny + iy)];
                col[2 * ix + 1] = data[2 * ((size_t)ix * ny + iy) + 1];
            }
            orc_fft_exec(px, col, work, sign);
            for (int ix = 0; ix < nx; ix++) {
                data[2 * ((size_t)ix * ny + iy)] = col[2 * ix];
                data[2 * ((size_t)ix * ny + iy) + 1] = col[2 * ix + 1];
            }
        }
        free(work);
        free(col);
    }
    orc_fft_plan_destroy(px);
    orc_fft_plan_destroy(py);
    return 0;
}

/*
 * GFMDSolverStatic::post_force, src/solvers/gfmd_solver_static.cpp:145-249,
 * with GFMDSolverFFT::fft_forward/fft_reverse
 * (src/solvers/gfmd_solver_fft.cpp:96-147, 150-195) inlined, single process.
 */
static double post_force_impl(int nx, int ny, int ndof, const double *phi, int half,
                              const double *linf, const double *u, double *f,
                              double *u0, int nthreads)
{
    const size_t nxy = (size_t)nx * ny;
    const int nu = ndof / 3;
    if (nthreads <= 0) nthreads = orc_max_threads();

    /* q_buffer[idq][idim], complex AoS (gfmd_solver_fft.cpp:136-144) */
    double *q = (double *)malloc(sizeof(double) * 2 * nxy * (size_t)ndof);
    double *fft_data = (double *)malloc(sizeof(double) * 2 * nxy);

    /* u(r) -> u(q), one complex 2-D transform per degree of freedom */
    for (int idim = 0; idim < ndof; idim++) {
        for (size_t i = 0; i < nxy; i++) {
            fft_data[2 * i] = u[(size_t)idim * nxy + i];
            fft_data[2 * i + 1] = 0.0;
        }
        orc_fft2d(fft_data, nx, ny, 1, nthreads);
        for (size_t i = 0; i < nxy; i++) {
            q[2 * (i * ndof + idim)] = fft_data[2 * i];
            q[2 * (i * ndof + idim) + 1] = fft_data[2 * i + 1];
        }
    }

    /* q = 0 component (gfmd_solver_static.cpp:169-177) */
    if (u0)
        for (int idim = 0; idim < ndof; idim++) u0[idim] = q[2 * idim];

    /* gamma-point energy (gfmd_solver_static.cpp:193-197) */
    double epot = 0.0;
    if (linf)
        for (int i = 0; i < nu; i++) epot -= 2.0 * linf[i] * q[2 * (3 * i + 2)];

    /* F(q) = Phi(q) u(q); epot += Re(conj(F) u); q = -F (:203-209) */
    double esum = 0.0;
#pragma omp parallel for num_threads(nthreads) reduction(+ : esum) schedule(static)
    for (long idq = 0; idq < (long)nxy; idq++) {
        double Fr[24], Fi[24];
        const double *P;
        double cj = 1.0; /* -1: conjugate of the mirrored stored entry */
        if (!half) {
            P = phi + 2 * (size_t)idq * ndof * ndof;
        } else {
            const int nyc = ny / 2 + 1;
            const int ix = (int)(idq / ny), iy = (int)(idq % ny);
            if (iy < nyc) {
                P = phi + 2 * ((size_t)ix * nyc + iy) * ndof * ndof;
            } else {
                P = phi + 2 * ((size_t)((nx - ix) % nx) * nyc + (ny - iy)) * ndof * ndof;
                cj = -1.0;
            }
        }
        double *uq = q + 2 * (size_t)idq * ndof;
        for (int i = 0; i < ndof; i++) {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < ndof; j++) {
                double pr = P[2 * (i * ndof + j)], pi = cj * P[2 * (i * ndof + j) + 1];
                double xr = uq[2 * j], xi = uq[2 * j + 1];
                sr += pr * xr - pi * xi;
                si += pr * xi + pi * xr;
            }
            Fr[i] = sr;
            Fi[i] = si;
        }
        for (int i = 0; i < ndof; i++) {
            esum += Fr[i] * uq[2 * i] + Fi[i] * uq[2 * i + 1];
            uq[2 * i] = -Fr[i];
            uq[2 * i + 1] = -Fi[i];
        }
    }
    epot += esum;

    /* linear force at the gamma point (:228-231) */
    if (linf)
        for (int i = 0; i < nu; i++) q[2 * (3 * i + 2)] += linf[i];

    epot *= 0.5;

    /* f(q) -> f(r), keep the real part (gfmd_solver_fft.cpp:150-195) */
    for (int idim = 0; idim < ndof; idim++) {
        for (size_t i = 0; i < nxy; i++) {
            fft_data[2 * i] = q[2 * (i * ndof + idim)];
            fft_data[2 * i + 1] = q[2 * (i * ndof + idim) + 1];
        }
        orc_fft2d(fft_data, nx, ny, -1, nthreads);
        for (size_t i = 0; i < nxy; i++) f[(size_t)idim * nxy + i] = fft_data[2 * i];
    }

    free(fft_data);
    free(q);
    return epot;
}

double orc_post_force(int nx, int ny, int ndof, const double *phi,
                      const double *linf, const double *u, double *f,
                      double *u0, int nthreads)
{
    return post_force_impl(nx, ny, ndof, phi, 0, linf, u, f, u0, nthreads);
}

double orc_post_force_half(int nx, int ny, int ndof, const double *phi_half,
                           const double *linf, const double *u, double *f,
                           double *u0, int nthreads)
{
    return post_force_impl(nx, ny, ndof, phi_half, 1, linf, u, f, u0, nthreads);
}

/* SplitMix64 finaliser: a counter-based hash, so that every thread fills
 * its wavevectors independently and the table does not depend on the thread
 * count. */
static unsigned long long orc_mix64(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

static double orc_unit(unsigned long long seed, unsigned long long i)
{
    return (double)(orc_mix64(seed ^ orc_mix64(i)) >> 11) * (1.0 / 9007199254740992.0) - 0.5;
}

void orc_synthetic_phi_full(int nx, int ny, int ndof, unsigned long long seed, double scale,
                            double *full, int nthreads)
{
    const size_t d2 = (size_t)ndof * ndof;
    if (nthreads <= 0) nthreads = orc_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int ix = 0; ix < nx; ix++) {
        for (int iy = 0; iy < ny; iy++) {
            /* canonical member of the pair (q, -q): the mirror entry is the
             * complex conjugate, so Phi(-q) = conj Phi(q) holds exactly */
            const int mx = (nx - ix) % nx, my = (ny - iy) % ny;
            const long a = (long)ix * ny + iy, b = (long)mx * ny + my;
            const long c = a < b ? a : b;
            const double cj = (a <= b) ? 1.0 : -1.0;
            double *dst = full + 2 * (size_t)a * d2;
            for (int i = 0; i < ndof; i++) {
                for (int j = i; j < ndof; j++) {
                    const unsigned long long k = ((unsigned long long)c * d2 + (size_t)i * ndof + j) * 2;
                    double re = scale * orc_unit(seed, k);
                    double im = (i == j) ? 0.0 : cj * scale * orc_unit(seed, k + 1);
                    if (i == j) re += 2.0 * scale;
                    if (a == b) im = 0.0; /* self-mirror wavevectors: real */
                    dst[2 * (i * ndof + j)] = re;
                    dst[2 * (i * ndof + j) + 1] = im;
                    dst[2 * (j * ndof + i)] = re;
                    dst[2 * (j * ndof + i) + 1] = -im;
                }
            }
        }
    }
}

void orc_phi_half_to_full(int nx, int ny, int ndof, const double *half, double *full,
                          int nthreads)
{
    const int nyc = ny / 2 + 1;
    const size_t d2 = (size_t)ndof * ndof;
    if (nthreads <= 0) nthreads = orc_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int ix = 0; ix < nx; ix++) {
        for (int iy = 0; iy < ny; iy++) {
            double *dst = full + 2 * ((size_t)ix * ny + iy) * d2;
            if (iy < nyc) {
                memcpy(dst, half + 2 * ((size_t)ix * nyc + iy) * d2, sizeof(double) * 2 * d2);
            } else {
                int mx = (nx - ix) % nx, my = ny - iy;
                const double *src = half + 2 * ((size_t)mx * nyc + my) * d2;
                for (size_t e = 0; e < d2; e++) {
                    dst[2 * e] = src[2 * e];
                    dst[2 * e + 1] = -src[2 * e + 1];
                }
            }
        }
    }
}
