/* steps_oracle.c -- TEST ORACLE ONLY (see steps_oracle.h).
 *
 * A plain-C restatement of the reference StePS CPU direct-summation path.
 * Each function names the reference file:line it follows (paths relative to
 * the StePS project root). It mirrors the reference's arithmetic (pow-based
 * spline, sequential-in-j accumulation per i, OpenMP over i with per-pair
 * atomic adds as forces.cc:550-555 does) so that it is both a tight numerical
 * pin and a like-for-like CPU timing baseline. Pinned against the reference
 * compiled from source (oracle/_ref) by tests/test_oracle_ref.py, and against
 * the golden vectors it produced by tests/test_oracle_golden.py.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library; the product library never does.
 */
#include "steps_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PI 3.14159265358979323846264338327950288419716939937510
#define ORACLE_SQRTPI 1.7724538509055160272981674833411

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

/* Cubic-spline softened force coefficient w(r, beta): forces.cc:52-87.
 * r >= beta: 1/r^3; beta/2 < r < beta: outer spline shell; else inner core. */
double oracle_force_softening(double r, double beta)
{
    double half = beta * 0.5;
    if (r >= beta) return pow(r, -3);
    if (r > half && r < beta) {
        double c0 = -32.0 / (3.0 * pow(beta, 6));
        double c1 = 38.4 / pow(beta, 5);
        double c2 = -48.0 / pow(beta, 4);
        double c3 = 64.0 / (3.0 * pow(beta, 3));
        double c4 = -1.0 / 15.0;
        return c0 * pow(r, 3) + c1 * pow(r, 2) + c2 * r + c3 + c4 / pow(r, 3);
    }
    {
        double c0 = 32.0 / pow(beta, 6);
        double c1 = -38.4 / pow(beta, 5);
        double c2 = 32.0 / (3.0 * pow(beta, 3));
        return c0 * pow(r, 3) + c1 * pow(r, 2) + c2;
    }
}

static void add_background(const oracle_params *p, const double *xi, double *Fi, int axes)
{
    /* forces.cc:557-568 (R^3, axes = 3) and :1293-1304 (S1xR2 x,y only, axes = 2). */
    if (p->cosmology == 1 && p->comoving == 1) {
        for (int k = 0; k < axes; k++) Fi[k] += p->mass_in_unit_sphere * xi[k];
    } else if (p->cosmology == 1 && p->comoving == 0) {
        double de = p->h0 * p->h0 * p->omega_lambda;
        for (int k = 0; k < axes; k++) Fi[k] += de * xi[k];
    }
}

static int dyn_chunk(int id_min, int id_max)
{
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    int c = (id_max - id_min) / nt;
    return c < 1 ? 1 : c;
}

/* R^3 direct sum: forces.cc:510-577. */
void oracle_forces_r3(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                      const oracle_params *p, double *F)
{
    int ni = id_max - id_min + 1;
    for (int q = 0; q < 3 * ni; q++) F[q] = 0.0;
    int chunk = dyn_chunk(id_min, id_max);
#pragma omp parallel for schedule(dynamic, chunk)
    for (int i = id_min; i <= id_max; i++) {
        double *Fi = F + 3 * (i - id_min);
        for (int j = 0; j < n; j++) {
            double b = eps[i] + eps[j];
            double dx = x[3 * j] - x[3 * i];
            double dy = x[3 * j + 1] - x[3 * i + 1];
            double dz = x[3 * j + 2] - x[3 * i + 2];
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double w = m[j] * oracle_force_softening(r, b);
#pragma omp atomic
            Fi[0] += w * dx;
#pragma omp atomic
            Fi[1] += w * dy;
#pragma omp atomic
            Fi[2] += w * dz;
        }
        add_background(p, x + 3 * i, Fi, 3);
    }
}

/* ---------------- T^3 ---------------- */

static int pos_mod(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

/* Cell-centred grid mapping: ewald_space.cc:398-406. */
static void centred_cell(double r, double L, int ng, int *i0, double *f)
{
    double h = L / (double)ng;
    double u = (r + L * 0.5) / h - 0.5;
    double uf = floor(u);
    *i0 = pos_mod((int)uf, ng);
    *f = u - uf;
}

/* Catmull-Rom cubic weights (order 4): ewald_space.cc:440-449;
 * 2-point Lagrange (order 2): ewald_space.cc:409-438 with stencil 2. */
static void interp_weights(double t, int order, double *w)
{
    if (order == 4) {
        double t2 = t * t, t3 = t * t2;
        w[0] = -0.5 * t3 + t2 - 0.5 * t;
        w[1] = 1.5 * t3 - 2.5 * t2 + 1.0;
        w[2] = -1.5 * t3 + 2.0 * t2 + 0.5 * t;
        w[3] = 0.5 * t3 - 0.5 * t2;
    } else {
        w[0] = (t - 1.0) / (0.0 - 1.0);
        w[1] = (t - 0.0) / (1.0 - 0.0);
    }
}

/* Tensor-product table interpolation of D(dx,dy,dz): ewald_space.cc:452-523. */
void oracle_t3_interp(int ngrid, double L, const double *table, double dx, double dy, double dz, int order,
                      double D[3])
{
    if (order != 4) order = 2;
    int ix0, iy0, iz0;
    double fx, fy, fz, wx[4], wy[4], wz[4];
    centred_cell(dx, L, ngrid, &ix0, &fx);
    centred_cell(dy, L, ngrid, &iy0, &fy);
    centred_cell(dz, L, ngrid, &iz0, &fz);
    interp_weights(fx, order, wx);
    interp_weights(fy, order, wy);
    interp_weights(fz, order, wz);
    int off = -(order / 2 - 1);
    double s0 = 0, s1 = 0, s2 = 0;
    for (int a = 0; a < order; a++) {
        int ix = pos_mod(ix0 + off + a, ngrid);
        for (int b = 0; b < order; b++) {
            int iy = pos_mod(iy0 + off + b, ngrid);
            double wxy = wx[a] * wy[b];
            for (int c = 0; c < order; c++) {
                int iz = pos_mod(iz0 + off + c, ngrid);
                double w = wxy * wz[c];
                size_t q = ((size_t)((ix * ngrid + iy) * ngrid + iz)) * 3u;
                s0 += w * table[q];
                s1 += w * table[q + 1];
                s2 += w * table[q + 2];
            }
        }
    }
    D[0] = s0;
    D[1] = s1;
    D[2] = s2;
}

static double nearest_image(double d, double L)
{
    /* forces.cc:812-817: subtract L*sign(d) once if |d| > L/2. */
    if (fabs(d) > 0.5 * L) d = d - L * d / fabs(d);
    return d;
}

/* T^3 direct sum + Ewald table correction: forces.cc:776-876. */
void oracle_forces_t3(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                      const oracle_params *p, const double *table, int ngrid, int order, double *F)
{
    int ni = id_max - id_min + 1;
    double L = p->L;
    for (int q = 0; q < 3 * ni; q++) F[q] = 0.0;
    int chunk = dyn_chunk(id_min, id_max);
    int ewald = p->is_periodic >= 2;
#pragma omp parallel for schedule(dynamic, chunk)
    for (int i = id_min; i <= id_max; i++) {
        double *Fi = F + 3 * (i - id_min);
        for (int j = 0; j < n; j++) {
            double b = eps[i] + eps[j];
            double dx = nearest_image(x[3 * j] - x[3 * i], L);
            double dy = nearest_image(x[3 * j + 1] - x[3 * i + 1], L);
            double dz = nearest_image(x[3 * j + 2] - x[3 * i + 2], L);
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double fx, fy, fz;
            if (ewald) {
                double w = oracle_force_softening(r, b);
                double D[3];
                oracle_t3_interp(ngrid, L, table, dx, dy, dz, order, D);
                fx = m[j] * (w * dx - D[0]);
                fy = m[j] * (w * dy - D[1]);
                fz = m[j] * (w * dz - D[2]);
            } else {
                double w = m[j] * oracle_force_softening(r, b);
                fx = w * dx;
                fy = w * dy;
                fz = w * dz;
            }
#pragma omp atomic
            Fi[0] += fx;
#pragma omp atomic
            Fi[1] += fy;
#pragma omp atomic
            Fi[2] += fz;
        }
    }
}

/* ---------------- S1 x R2 ---------------- */

/* Linear interpolation of the cylindrical background multiplier: forces.cc:279-316
 * with ORDER = 1 (abscissae step*i with step = R/size, index from r/R*(size-1)). */
double oracle_cyl_correction(double r, double R, const double *table, int size)
{
    double step = R / (double)size;
    int i = (int)floor(r / R * (size - 1));
    double c = table[size - 1];
    if (i < size - 1) {
        double x1 = step * i, y1 = table[i], x2 = step * (i + 1), y2 = table[i + 1];
        double A = (y2 - y1) / (x2 - x1);
        double B = y1 - A * x1;
        c = A * r + B;
    }
    return c;
}

static void add_background_cyl(const oracle_params *p, const double *xi, double *Fi, const double *radial,
                               int radial_size, int use_table)
{
    if (p->cosmology == 1 && p->comoving == 1) {
        double corr = 1.0;
        if (use_table) {
            double rxy = sqrt(xi[0] * xi[0] + xi[1] * xi[1]);
            corr = oracle_cyl_correction(rxy, p->rsim, radial, radial_size);
            Fi[0] += p->mass_in_unit_sphere * xi[0] * corr;
            Fi[1] += p->mass_in_unit_sphere * xi[1] * corr;
        } else {
            Fi[0] += p->mass_in_unit_sphere * xi[0];
            Fi[1] += p->mass_in_unit_sphere * xi[1];
        }
    } else if (p->cosmology == 1 && p->comoving == 0) {
        double de = p->h0 * p->h0 * p->omega_lambda;
        Fi[0] += de * xi[0];
        Fi[1] += de * xi[1];
    }
}

/* S1xR2 explicit image sum along z (PERIODIC_Z_NOLOOKUP): forces.cc:1250-1305,
 * and the quasi-periodic nearest-image case IS_PERIODIC == 1: forces.cc:1354-1397.
 * Images m in [-e, e], e = IS_PERIODIC+1, kept when |dz + mL| <= (e - 0.4) L
 * (main.cc:1270-1271). */
void oracle_forces_s1r2_images(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                               const oracle_params *p, const double *radial_table, int radial_size, double *F)
{
    int ni = id_max - id_min + 1;
    double L = p->L;
    for (int q = 0; q < 3 * ni; q++) F[q] = 0.0;
    int chunk = dyn_chunk(id_min, id_max);
    int emax = p->is_periodic + 1;
    double ecut = (double)emax - 0.4;
#pragma omp parallel for schedule(dynamic, chunk)
    for (int i = id_min; i <= id_max; i++) {
        double *Fi = F + 3 * (i - id_min);
        for (int j = 0; j < n; j++) {
            double b = eps[i] + eps[j];
            double dx = x[3 * j] - x[3 * i];
            double dy = x[3 * j + 1] - x[3 * i + 1];
            double dz = x[3 * j + 2] - x[3 * i + 2];
            double fx = 0, fy = 0, fz = 0;
            if (p->is_periodic >= 2) {
                for (int k = -emax; k < emax + 1; k++) {
                    double dzk = dz + ((double)k) * L;
                    double r = sqrt(dx * dx + dy * dy + dzk * dzk);
                    if (fabs(dzk) <= ecut * L) {
                        double w = m[j] * oracle_force_softening(r, b);
                        fx += w * dx;
                        fy += w * dy;
                        fz += w * dzk;
                    }
                }
            } else {
                if (fabs(dz) > 0.5 * L) dz = dz - L * dz / fabs(dz);
                double r = sqrt(dx * dx + dy * dy + dz * dz);
                double w = m[j] * oracle_force_softening(r, b);
                fx = w * dx;
                fy = w * dy;
                fz = w * dz;
            }
#pragma omp atomic
            Fi[0] += fx;
#pragma omp atomic
            Fi[1] += fy;
#pragma omp atomic
            Fi[2] += fz;
        }
        add_background_cyl(p, x + 3 * i, Fi, radial_table, radial_size, 1);
    }
}

static size_t cyl_off(int nz, int ir, int iz, int c) { return ((size_t)ir * (size_t)nz + (size_t)iz) * 2u + (size_t)c; }

/* (rho, z) table interpolation, orders 0 = NGP, 2 = CIC, 4 = TSC:
 * ewald_space.cc:803-1000, Cartesian mapping :1003-1048. */
void oracle_s1r2_interp(const double *T, int nrho, int nz, double rho_max, double lz, double dx, double dy, double dz,
                        int order, double D[3])
{
    double rho = sqrt(dx * dx + dy * dy);
    double Dr = 0, Dz = 0;
    double half = 0.5 * lz;
    double drho = rho_max / (double)(nrho - 1 > 1 ? nrho - 1 : 1);
    double dzc = lz / (double)nz;
    double rr = rho;
    if (order == 0) {
        if (rr < 0) rr = 0;
        if (rr > rho_max) rr = rho_max;
        double ur = drho > 0 ? rr / drho : 0.0;
        double uz = (dz + half) / dzc - 0.5;
        int ir = (int)floor(ur + 0.5);
        int iz = (int)floor(uz + 0.5);
        if (ir < 0) ir = 0;
        if (ir > nrho - 1) ir = nrho - 1;
        iz = pos_mod(iz, nz);
        Dr = T[cyl_off(nz, ir, iz, 0)];
        Dz = T[cyl_off(nz, ir, iz, 1)];
    } else if (order == 2) {
        rr = rr < 0 ? 0 : (rr > rho_max ? rho_max : rr);
        double ur = drho > 0 ? rr / drho : 0.0;
        int ir0 = (int)floor(ur);
        double fr = ur - (double)ir0;
        if (ir0 < 0) { ir0 = 0; fr = 0; }
        if (ir0 > nrho - 2) { ir0 = nrho - 2 > 0 ? nrho - 2 : 0; fr = 1.0; }
        int ir1 = ir0 + 1;
        double uz = (dz + half) / dzc - 0.5;
        int iz0 = (int)floor(uz);
        double fz = uz - (double)iz0;
        iz0 = pos_mod(iz0, nz);
        int iz1 = pos_mod(iz0 + 1, nz);
        double w00 = 1.0 - fr; w00 *= (1.0 - fz);
        double w10 = fr; w10 *= (1.0 - fz);
        double w01 = 1.0 - fr; w01 *= fz;
        double w11 = fr * fz;
        Dr = w00 * T[cyl_off(nz, ir0, iz0, 0)] + w10 * T[cyl_off(nz, ir1, iz0, 0)] + w01 * T[cyl_off(nz, ir0, iz1, 0)] +
             w11 * T[cyl_off(nz, ir1, iz1, 0)];
        Dz = w00 * T[cyl_off(nz, ir0, iz0, 1)] + w10 * T[cyl_off(nz, ir1, iz0, 1)] + w01 * T[cyl_off(nz, ir0, iz1, 1)] +
             w11 * T[cyl_off(nz, ir1, iz1, 1)];
    } else {
        if (rr < 0) rr = 0;
        if (rr > rho_max) rr = rho_max;
        double ur = drho > 0 ? rr / drho : 0.0;
        double uz = (dz + half) / dzc - 0.5;
        int jr = (int)floor(ur + 0.5);
        int jz = (int)floor(uz + 0.5);
        double sr = ur - (double)jr, sz = uz - (double)jz;
        double wr[3] = {0.5 * (0.5 - sr) * (0.5 - sr), 0.75 - sr * sr, 0.5 * (0.5 + sr) * (0.5 + sr)};
        double wz[3] = {0.5 * (0.5 - sz) * (0.5 - sz), 0.75 - sz * sz, 0.5 * (0.5 + sz) * (0.5 + sz)};
        int ir[3] = {jr - 1, jr, jr + 1};
        if (ir[0] < 0) ir[0] = 0;
        if (ir[1] < 0) ir[1] = 0;
        if (ir[1] > nrho - 1) ir[1] = nrho - 1;
        if (ir[2] > nrho - 1) ir[2] = nrho - 1;
        int izs[3] = {pos_mod(jz - 1, nz), pos_mod(jz, nz), pos_mod(jz + 1, nz)};
        for (int zr = 0; zr < 3; zr++) {
            double w0 = wr[0] * wz[zr], w1 = wr[1] * wz[zr], w2 = wr[2] * wz[zr];
            Dr += w0 * T[cyl_off(nz, ir[0], izs[zr], 0)] + w1 * T[cyl_off(nz, ir[1], izs[zr], 0)] +
                  w2 * T[cyl_off(nz, ir[2], izs[zr], 0)];
            Dz += w0 * T[cyl_off(nz, ir[0], izs[zr], 1)] + w1 * T[cyl_off(nz, ir[1], izs[zr], 1)] +
                  w2 * T[cyl_off(nz, ir[2], izs[zr], 1)];
        }
    }
    double ex = rho > 0 ? dx / rho : 0.0;
    double ey = rho > 0 ? dy / rho : 0.0;
    D[0] = Dr * ex;
    D[1] = Dr * ey;
    D[2] = Dz;
}

/* S1xR2 nearest image + (rho,z) table correction: forces.cc:1307-1350. */
void oracle_forces_s1r2_table(int n, const double *x, const double *m, const double *eps, int id_min, int id_max,
                              const oracle_params *p, const double *table, int nrho, int nz, int order,
                              const double *radial_table, int radial_size, double *F)
{
    if (p->is_periodic < 2) {
        oracle_forces_s1r2_images(n, x, m, eps, id_min, id_max, p, radial_table, radial_size, F);
        return;
    }
    int ni = id_max - id_min + 1;
    double L = p->L;
    double rho_max = 2.25 * p->rsim; /* EWALD_LOOKUP_TABLE_RADIAL_EXTENT_FACTOR, global_variables.h:39 */
    for (int q = 0; q < 3 * ni; q++) F[q] = 0.0;
    int chunk = dyn_chunk(id_min, id_max);
#pragma omp parallel for schedule(dynamic, chunk)
    for (int i = id_min; i <= id_max; i++) {
        double *Fi = F + 3 * (i - id_min);
        for (int j = 0; j < n; j++) {
            double b = eps[i] + eps[j];
            double dx = x[3 * j] - x[3 * i];
            double dy = x[3 * j + 1] - x[3 * i + 1];
            double dz = x[3 * j + 2] - x[3 * i + 2];
            if (fabs(dz) > 0.5 * L) dz = dz - L * dz / fabs(dz);
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double w = oracle_force_softening(r, b);
            double D[3];
            oracle_s1r2_interp(table, nrho, nz, rho_max, L, dx, dy, dz, order, D);
            double fx = m[j] * (w * dx - D[0]);
            double fy = m[j] * (w * dy - D[1]);
            double fz = m[j] * (w * dz - D[2]);
#pragma omp atomic
            Fi[0] += fx;
#pragma omp atomic
            Fi[1] += fy;
#pragma omp atomic
            Fi[2] += fz;
        }
        add_background_cyl(p, x + 3 * i, Fi, radial_table, radial_size, 0);
    }
}

/* ---------------- Ewald table builders ---------------- */

/* Integer lattice points with i^2+j^2+k^2 < R^2 and |i|,|j|,|k| < R, in the
 * enumeration order of ewald_space() (ewald_space.cc:118-205). Returns the
 * number of points (the reference returns that number minus one). */
int oracle_lattice(double R, int *out, int cap)
{
    int l = 0;
#define PUT(a, b, c)                                                                                                   \
    do {                                                                                                               \
        if (l < cap) {                                                                                                 \
            out[4 * l] = (a); out[4 * l + 1] = (b); out[4 * l + 2] = (c); out[4 * l + 3] = i * i + j * j + k * k;       \
        }                                                                                                              \
        l++;                                                                                                           \
    } while (0)
    for (int i = 0; i < R; i++)
        for (int j = 0; j < R; j++)
            for (int k = 0; k < R; k++) {
                if (!((double)(i * i + j * j + k * k) < R * R)) continue;
                PUT(i, j, k);
                if (i) PUT(-i, j, k);
                if (j) PUT(i, -j, k);
                if (k) PUT(i, j, -k);
                if (j && k) PUT(i, -j, -k);
                if (i && k) PUT(-i, j, -k);
                if (i && j) PUT(-i, -j, k);
                if (i && j && k) PUT(-i, -j, -k);
            }
#undef PUT
    return l;
}

/* Ewald correction D(r) = F_real + F_recip - F_Newton(nearest image):
 * ewald_space.cc:210-286 (Hernquist, Bouchet & Suto 1991 Ewald sums). */
static void t3_correction(const double r[3], double L, double alpha, int nreal, const int *real_idx, int nrec,
                          const int *rec_idx, double rel_cut, double rec_cut, double D[3])
{
    double Fr[3] = {0, 0, 0}, Fk[3] = {0, 0, 0};
    double V = L * L * L;
    double c_gauss = 2.0 * alpha / sqrt(ORACLE_PI);
    double c_rec = (4.0 * ORACLE_PI) / V;
    double relcut2 = (rel_cut * L) * (rel_cut * L);
    for (int q = 0; q < nreal; q++) {
        double R[3] = {r[0] + (double)real_idx[4 * q] * L, r[1] + (double)real_idx[4 * q + 1] * L,
                       r[2] + (double)real_idx[4 * q + 2] * L};
        double R2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
        if (R2 == 0.0 || R2 > relcut2) continue;
        double Rn = sqrt(R2);
        double inv = 1.0 / Rn;
        double inv3 = inv * inv * inv;
        double br = erfc(alpha * Rn) + c_gauss * Rn * exp(-(alpha * alpha) * R2);
        double co = inv3 * br;
        Fr[0] += -R[0] * co;
        Fr[1] += -R[1] * co;
        Fr[2] += -R[2] * co;
    }
    for (int q = 0; q < nrec; q++) {
        int hx = rec_idx[4 * q], hy = rec_idx[4 * q + 1], hz = rec_idx[4 * q + 2];
        if (hx == 0 && hy == 0 && hz == 0) continue;
        double f = 2.0 * ORACLE_PI / L;
        double kv[3] = {f * (double)hx, f * (double)hy, f * (double)hz};
        double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        if (k2 == 0.0 || k2 > rec_cut * rec_cut) continue;
        double damp = exp(-k2 / (4.0 * alpha * alpha));
        double co = c_rec * damp / k2;
        double s = sin(kv[0] * r[0] + kv[1] * r[1] + kv[2] * r[2]);
        Fk[0] += -kv[0] * co * s;
        Fk[1] += -kv[1] * co * s;
        Fk[2] += -kv[2] * co * s;
    }
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    if (r2 > 0.0) {
        double rn = sqrt(r2);
        double i3 = 1.0 / (rn * rn * rn);
        for (int c = 0; c < 3; c++) D[c] = (Fr[c] + Fk[c]) - (-r[c] * i3);
    } else {
        D[0] = D[1] = D[2] = 0.0;
    }
}

/* The 24 proper rotations of the cube (group O) as signed axis permutations,
 * in the order ewald_space.cc:64-98 lists them: even permutations with an even
 * number of sign flips, then odd permutations with an odd number. */
static void cube_rotations(int perm[24][3], int sgn[24][3])
{
    static const int pe[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    static const int po[3][3] = {{0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
    static const int sp[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
    static const int sn[4][3] = {{-1, -1, -1}, {-1, 1, 1}, {1, -1, 1}, {1, 1, -1}};
    int q = 0;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 4; b++, q++)
            for (int k = 0; k < 3; k++) { perm[q][k] = pe[a][k]; sgn[q][k] = sp[b][k]; }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 4; b++, q++)
            for (int k = 0; k < 3; k++) { perm[q][k] = po[a][k]; sgn[q][k] = sn[b][k]; }
}

/* T^3 table on the cell-centred ngrid^3 grid over [-L/2, L/2]^3:
 * ewald_space.cc:288-383 (wedge x >= y >= z >= 0, filled out by the 24
 * rotations and the inversion). Index sets as main.cc:467-468 builds them:
 * lattice(real_radius) for the real sum, lattice(rec_radius) for k. */
void oracle_t3_table(int ngrid, double L, double alpha, double rel_cut, double rec_cut, double real_radius,
                     double rec_radius, double *out)
{
    int cap = 60000;
    int *ri = (int *)malloc(sizeof(int) * 4 * (size_t)cap);
    int *ki = (int *)malloc(sizeof(int) * 4 * (size_t)cap);
    int nreal = oracle_lattice(real_radius, ri, cap);
    int nrec = oracle_lattice(rec_radius, ki, cap);
    if (nreal > cap) nreal = cap;
    if (nrec > cap) nrec = cap;
    int perm[24][3], sgn[24][3];
    cube_rotations(perm, sgn);
    memset(out, 0, sizeof(double) * 3 * (size_t)ngrid * ngrid * ngrid);
    double h = L / (double)ngrid;
    int c0 = ngrid / 2;
#define TAB(a, b, c, comp) out[((size_t)(((a) * ngrid + (b)) * ngrid + (c))) * 3u + (comp)]
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = c0; i < ngrid; i++)
        for (int j = c0; j <= i; j++)
            for (int k = c0; k <= j; k++) {
                double r[3] = {((double)i + 0.5) * h - L / 2.0, ((double)j + 0.5) * h - L / 2.0,
                               ((double)k + 0.5) * h - L / 2.0};
                double Dw[3];
                t3_correction(r, L, alpha, nreal, ri, nrec, ki, rel_cut, rec_cut, Dw);
                for (int c = 0; c < 3; c++) TAB(i, j, k, c) = Dw[c];
                int src[3] = {i, j, k};
                for (int q = 0; q < 24; q++) {
                    int dst[3];
                    double Dr[3];
                    for (int d = 0; d < 3; d++) {
                        int v = src[perm[q][d]];
                        if (sgn[q][d] < 0) v = (ngrid - 1) - v;
                        dst[d] = v;
                        Dr[d] = sgn[q][d] * Dw[perm[q][d]];
                    }
                    for (int c = 0; c < 3; c++) TAB(dst[0], dst[1], dst[2], c) = Dr[c];
                    int inv0 = (ngrid - 1) - dst[0], inv1 = (ngrid - 1) - dst[1], inv2 = (ngrid - 1) - dst[2];
                    for (int c = 0; c < 3; c++) TAB(inv0, inv1, inv2, c) = -Dr[c];
                }
            }
#undef TAB
    free(ri);
    free(ki);
}

/* Scaled complementary error function erfcx(x) = exp(x^2) erfc(x) by the
 * Abramowitz & Stegun 7.1.26 rational fit, as ewald_space.cc:537-561 uses it. */
static double as_erfcx(double x)
{
    if (x < 0) return 2.0 * exp(x * x) - as_erfcx(-x);
    if (x == 0) return 1.0;
    if (x > 1e10) return 0.564189583547756286 / x;
    double t = 1.0 / (1.0 + 0.3275911 * x);
    return t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))));
}

/* exp(+-k rho) erfc(k/(2 alpha) +- alpha rho) without overflow: ewald_space.cc:564-596. */
static double exp_erfc(double km, double rho, double alpha, int plus)
{
    double a2 = km / (2.0 * alpha);
    double ar = alpha * rho;
    double arg = plus ? (a2 + ar) : (a2 - ar);
    double common = -(a2 * a2 + ar * ar);
    if (arg > 5.0) return exp(common) * as_erfcx(arg);
    if (arg < -5.0) return 2.0 * exp(-km * rho) - exp(common) * as_erfcx(-arg);
    return exp(plus ? km * rho : -km * rho) * erfc(arg);
}

/* Nearest-image wrap of dz used by the S1xR2 builder: ewald_space.cc:600-609. */
static double wrap_dz(double dz, double lz)
{
    double half = 0.5 * lz;
    if (dz > half) dz -= lz * floor((dz + half) / lz);
    if (dz <= -half) dz -= lz * floor((dz - half) / lz);
    return dz;
}

/* Singly periodic (S1xR2) Ewald force per unit G m_i m_j, Tornberg (2015):
 * ewald_space.cc:618-752 (real-space images |n| <= nmax, modes m = 1..mmax,
 * and the m = 0 radial term). */
/* Direct real-space image sum with no k-space part: the reference's
 * PERIODIC_Z_RSPACELOOKUP build of S1R2ewald_force_pair (ewald_space.cc:710-750),
 * n = 0 first, then -n and +n for n = 1..nmax (largest terms first). That
 * build passes alpha = 0 and mmax = 0 (main.cc:650, :683), which select it here;
 * the Ewald sums below reduce to the same terms at those arguments, in
 * another order. */
static void s1r2_pair_direct(double dx, double dy, double dz, double rho2, double lz, int nmax, double F[3])
{
    double Fx = 0, Fy = 0, Fz = 0;
    double r2 = rho2 + dz * dz;
    if (r2 >= 1e-18) {
        double r = sqrt(r2);
        double invr3 = 1.0 / (r2 * r);
        Fx -= dx * invr3;
        Fy -= dy * invr3;
        Fz -= dz * invr3;
    }
    for (int n = 1; n <= nmax; ++n)
        for (int sign = -1; sign <= 1; sign += 2) {
            double dzn = dz + (double)(sign * n) * lz;
            r2 = rho2 + dzn * dzn;
            if (r2 < 1e-18) continue;
            double r = sqrt(r2);
            double invr3 = 1.0 / (r2 * r);
            Fx -= dx * invr3;
            Fy -= dy * invr3;
            Fz -= dzn * invr3;
        }
    F[0] = Fx;
    F[1] = Fy;
    F[2] = Fz;
}

void oracle_s1r2_pair(double dx, double dy, double dz, double lz, double alpha, int nmax, int mmax, double F[3])
{
    dz = wrap_dz(dz, lz);
    double rho2 = dx * dx + dy * dy;
    if (alpha == 0.0 && mmax == 0) {
        s1r2_pair_direct(dx, dy, dz, rho2, lz, nmax, F);
        return;
    }
    double rho = sqrt(rho2);
    double Fxr = 0, Fyr = 0, Fzr = 0;
    for (int n = -nmax; n <= nmax; ++n) {
        double dzn = dz + (double)n * lz;
        double r2 = rho2 + dzn * dzn;
        if (r2 < 1e-18) continue;
        double r = sqrt(r2);
        double invr3 = 1.0 / (r2 * r);
        double ar = alpha * r;
        double co = (erfc(ar) + (2.0 / ORACLE_SQRTPI) * ar * exp(-ar * ar)) * invr3;
        Fxr -= dx * co;
        Fyr -= dy * co;
        Fzr -= dzn * co;
    }
    double Frk = 0, Fzk = 0;
    double invL = 1.0 / lz;
    for (int m = 1; m <= mmax; ++m) {
        double km = (2.0 * ORACLE_PI * m) * invL;
        double tp = exp_erfc(km, rho, alpha, 1);
        double tm = exp_erfc(km, rho, alpha, 0);
        double B = tp + tm;
        double dB = km * (tp - tm);
        Frk += (2.0 * invL) * cos(km * dz) * dB;
        Fzk -= (2.0 * invL) * km * sin(km * dz) * B;
    }
    if (rho > 1e-12) Frk += -(2.0 * invL / rho) * (1.0 - exp(-alpha * alpha * rho2));
    double Fxk = rho > 0 ? Frk * dx / rho : 0.0;
    double Fyk = rho > 0 ? Frk * dy / rho : 0.0;
    F[0] = Fxr + Fxk;
    F[1] = Fyr + Fyk;
    F[2] = Fzr + Fzk;
}

/* (rho, z) correction table: ewald_space.cc:754-798. */
void oracle_s1r2_table(int nrho, int nz, double rho_max, double lz, double alpha, int nmax, int mmax, double *out)
{
    double drho = rho_max / (double)(nrho - 1 > 1 ? nrho - 1 : 1);
    double dzc = lz / (double)nz;
#pragma omp parallel for schedule(dynamic, 1)
    for (int ir = 0; ir < nrho; ++ir) {
        double rho = (double)ir * drho;
        for (int iz = 0; iz < nz; ++iz) {
            double z = ((double)iz + 0.5) * dzc - 0.5 * lz;
            double Fp[3];
            oracle_s1r2_pair(rho, 0.0, z, lz, alpha, nmax, mmax, Fp);
            double zw = wrap_dz(z, lz);
            double r2 = rho * rho + zw * zw;
            double Frn = 0, Fzn = 0;
            if (r2 > 0) {
                double r = sqrt(r2);
                double i3 = 1.0 / (r * r * r);
                Frn = -rho * i3;
                Fzn = -zw * i3;
            }
            out[cyl_off(nz, ir, iz, 0)] = Fp[0] - Frn;
            out[cyl_off(nz, ir, iz, 1)] = Fp[2] - Fzn;
        }
    }
}

/* Finite-cylinder radial background multiplier by the trapezoid rule: utils.cc:162-228. */
static double cyl_log_term(double lz, double R, double a, double Y, int plus)
{
    double s = sqrt(R * R - Y * Y);
    double sg = plus ? 2.0 * a * s : -2.0 * a * s;
    return sqrt(lz * lz + R * R + a * a + sg) + lz;
}

void oracle_cyl_table(double R, double lz, int size, int accuracy, double *out)
{
    double step = R / (double)accuracy;
    out[0] = 0.0;
    for (int i = 1; i < size; i++) {
        double a = (i == size - 1) ? R : R / (double)(size - 1) * i;
        double total = 0;
        for (int j = 1; j <= accuracy; j++) {
            double ip, in;
            if (a >= R) {
                a = R;
                double Y0 = (j - 1) * step, Y1 = j * step;
                ip = -2 * log(cyl_log_term(lz, R, R, Y0, 1) / cyl_log_term(lz, R, R, Y0, 0));
                in = -2 * log(cyl_log_term(lz, R, R, Y1, 1) / cyl_log_term(lz, R, R, Y1, 0));
            } else {
                double Y0 = (j - 1) * step, Y1 = j * step;
                double s0 = sqrt(R * R - Y0 * Y0), s1 = sqrt(R * R - Y1 * Y1);
                ip = -2 * log(cyl_log_term(lz, R, a, Y0, 1) / cyl_log_term(lz, R, a, Y0, 0)) +
                     log((R * R + a * a + 2 * a * s0) / (R * R + a * a - 2 * a * s0));
                in = -2 * log(cyl_log_term(lz, R, a, Y1, 1) / cyl_log_term(lz, R, a, Y1, 0)) +
                     log((R * R + a * a + 2 * a * s1) / (R * R + a * a - 2 * a * s1));
            }
            total += step * (ip + in) * 0.5;
        }
        if (a >= R)
            out[i] = 2 * (total + ORACLE_PI * R) / (2 * ORACLE_PI * R);
        else
            out[i] = 2 * total / (2 * ORACLE_PI * a);
    }
    if (size >= 3) {
        double x1 = 2 * R / (double)size, y1 = out[1], x2 = 4 * R / (double)size, y2 = out[2];
        double A = (y2 - y1) / (x2 - x1);
        out[0] = y1 - A * x1;
    }
}

/* ---------------- dispatch + KDK ---------------- */

void oracle_forces(const oracle_system *s, const double *x, int id_min, int id_max, double *F)
{
    switch (s->topology) {
    case 0: oracle_forces_r3(s->n, x, s->m, s->eps, id_min, id_max, &s->p, F); break;
    case 1: oracle_forces_t3(s->n, x, s->m, s->eps, id_min, id_max, &s->p, s->table, s->ngrid, s->order, F); break;
    case 2:
        oracle_forces_s1r2_table(s->n, x, s->m, s->eps, id_min, id_max, &s->p, s->table, s->nrho, s->nz, s->order,
                                 s->radial_table, s->radial_size, F);
        break;
    default:
        oracle_forces_s1r2_images(s->n, x, s->m, s->eps, id_min, id_max, &s->p, s->radial_table, s->radial_size, F);
        break;
    }
}

/* Fixed-h KDK (step.cc:100-312): kick h/2 + drift h, periodic wrap
 * (step.cc:151-180), force, kick h/2, errmax (step.cc:256-269). */
double oracle_kdk(const oracle_system *s, int nsteps, double h, double g, double a, double hubble, double rho_part,
                  double *x, double *v, double *F)
{
    int n = s->n;
    double a3 = pow(a, -3.0);
    double errmax = 0.0;
    double cb = 3.0 / rho_part / (4.0 * ORACLE_PI);
    for (int st = 0; st < nsteps; st++) {
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                double acc = g * F[3 * i + k] * a3 - 2.0 * hubble * v[3 * i + k];
                v[3 * i + k] += acc * (h / 2.0);
                x[3 * i + k] = x[3 * i + k] + v[3 * i + k] * h;
            }
        if (s->topology == 1) {
            for (int i = 0; i < 3 * n; i++) {
                if (x[i] < 0) x[i] += s->p.L;
                else if (x[i] >= s->p.L) x[i] -= s->p.L;
            }
        } else if (s->topology >= 2) {
            for (int i = 0; i < n; i++) {
                if (x[3 * i + 2] < 0) x[3 * i + 2] += s->p.L;
                else if (x[3 * i + 2] >= s->p.L) x[3 * i + 2] -= s->p.L;
            }
        }
        oracle_forces(s, x, 0, n - 1, F);
        errmax = 0.0;
        for (int i = 0; i < n; i++) {
            double acc[3];
            for (int k = 0; k < 3; k++) {
                acc[k] = g * F[3 * i + k] * a3 - 2.0 * hubble * v[3 * i + k];
                v[3 * i + k] += acc[k] * (h / 2.0);
            }
            double e = sqrt(acc[0] * acc[0] + acc[1] * acc[1] + acc[2] * acc[2]) / cbrt(s->m[i] * cb);
            if (e > errmax) errmax = e;
        }
    }
    return errmax;
}
