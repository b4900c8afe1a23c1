// Ewald correction tables built on the GPU in FP64.
//
// T^3 (StePS/src/ewald_space.cc:118-383): D(r) = F_real(r) + F_recip(r) -
// F_Newton(r) on the cell-centred ngrid^3 grid over [-L/2, L/2]^3, following
// Hernquist, Bouchet & Suto (1991). As in the reference, only the wedge
// x >= y >= z >= 0 is evaluated (one thread per wedge point) and the value is
// written to the 48 images of the point under the cube's symmetry group
// (24 rotations and the inversion, applied in the reference's order, so the
// table is symmetric exactly as the reference's is).
//
// S1xR2 (StePS/src/ewald_space.cc:539-798): the singly periodic Ewald sum of
// Tornberg (2015) minus the nearest-image Newtonian force on a (rho, z) grid.
// erfc/exp/sin/cos are CUDA's FP64 functions; erfcx for large arguments is
// the Abramowitz & Stegun 7.1.26 rational fit the reference uses.
#include <math.h>

#include <vector>

#include "common.cuh"
#include "context.cuh"

namespace steps {

namespace {

constexpr double PI = 3.14159265358979323846264338327950288419716939937510;

// Integer lattice points with |i|,|j|,|k| < R and i^2+j^2+k^2 < R^2, in the
// enumeration order of ewald_space() (StePS/src/ewald_space.cc:118-205).
std::vector<int4> lattice(double R)
{
    std::vector<int4> out;
    for (int i = 0; i < R; i++)
        for (int j = 0; j < R; j++)
            for (int k = 0; k < R; k++) {
                if (!((double)(i * i + j * j + k * k) < R * R)) continue;
                out.push_back(make_int4(i, j, k, 0));
                if (i) out.push_back(make_int4(-i, j, k, 0));
                if (j) out.push_back(make_int4(i, -j, k, 0));
                if (k) out.push_back(make_int4(i, j, -k, 0));
                if (j && k) out.push_back(make_int4(i, -j, -k, 0));
                if (i && k) out.push_back(make_int4(-i, j, -k, 0));
                if (i && j) out.push_back(make_int4(-i, -j, k, 0));
                if (i && j && k) out.push_back(make_int4(-i, -j, -k, 0));
            }
    return out;
}

struct Rotations {
    int perm[24][3];
    int sgn[24][3];
};

// The 24 proper rotations of the cube as signed axis permutations, listed as
// in StePS/src/ewald_space.cc:64-98: even permutations with an even number of
// sign flips, then odd permutations with an odd number.
Rotations cube_rotations()
{
    static const int pe[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
    static const int po[3][3] = {{0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
    static const int sp[4][3] = {{1, 1, 1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
    static const int sn[4][3] = {{-1, -1, -1}, {-1, 1, 1}, {1, -1, 1}, {1, 1, -1}};
    Rotations r;
    int q = 0;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 4; b++, q++)
            for (int k = 0; k < 3; k++) { r.perm[q][k] = pe[a][k]; r.sgn[q][k] = sp[b][k]; }
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 4; b++, q++)
            for (int k = 0; k < 3; k++) { r.perm[q][k] = po[a][k]; r.sgn[q][k] = sn[b][k]; }
    return r;
}

__global__ void k_t3_table(int ng, double L, double alpha, const int4 *__restrict__ real_idx, int nreal,
                           const int4 *__restrict__ rec_idx, int nrec, double rel_cut, double rec_cut, Rotations rot,
                           double *__restrict__ tab)
{
    const int c0 = ng / 2;
    const int span = ng - c0;
    long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)span * span * span) return;
    int i = c0 + (int)(id / ((long long)span * span));
    int j = c0 + (int)((id / span) % span);
    int k = c0 + (int)(id % span);
    if (!(j <= i && k <= j)) return;  // wedge x >= y >= z >= 0

    const double h = L / (double)ng;
    const double r[3] = {((double)i + 0.5) * h - L / 2.0, ((double)j + 0.5) * h - L / 2.0,
                         ((double)k + 0.5) * h - L / 2.0};
    double Fr[3] = {0, 0, 0}, Fk[3] = {0, 0, 0};
    const double c_gauss = 2.0 * alpha / sqrt(PI);
    const double c_rec = (4.0 * PI) / (L * L * L);
    const double relcut2 = (rel_cut * L) * (rel_cut * L);
    for (int q = 0; q < nreal; q++) {
        int4 n = real_idx[q];
        double R[3] = {r[0] + (double)n.x * L, r[1] + (double)n.y * L, r[2] + (double)n.z * L};
        double R2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
        if (R2 == 0.0 || R2 > relcut2) continue;
        double Rn = sqrt(R2);
        double inv = 1.0 / Rn;
        double co = inv * inv * inv * (erfc(alpha * Rn) + c_gauss * Rn * exp(-(alpha * alpha) * R2));
        Fr[0] += -R[0] * co;
        Fr[1] += -R[1] * co;
        Fr[2] += -R[2] * co;
    }
    const double f = 2.0 * PI / L;
    for (int q = 0; q < nrec; q++) {
        int4 hh = rec_idx[q];
        if (hh.x == 0 && hh.y == 0 && hh.z == 0) continue;
        double kv[3] = {f * (double)hh.x, f * (double)hh.y, f * (double)hh.z};
        double k2 = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
        if (k2 == 0.0 || k2 > rec_cut * rec_cut) continue;
        double co = c_rec * exp(-k2 / (4.0 * alpha * alpha)) / k2;
        double s = sin(kv[0] * r[0] + kv[1] * r[1] + kv[2] * r[2]);
        Fk[0] += -kv[0] * co * s;
        Fk[1] += -kv[1] * co * s;
        Fk[2] += -kv[2] * co * s;
    }
    double D[3] = {0, 0, 0};
    double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    if (r2 > 0.0) {
        double rn = sqrt(r2);
        double i3 = 1.0 / (rn * rn * rn);
        for (int c = 0; c < 3; c++) D[c] = (Fr[c] + Fk[c]) - (-r[c] * i3);
    }
    auto put = [&](int a, int b, int cc, const double *v) {
        double *o = tab + ((size_t)(a * ng + b) * ng + cc) * 3;
        o[0] = v[0];
        o[1] = v[1];
        o[2] = v[2];
    };
    put(i, j, k, D);
    const int src[3] = {i, j, k};
    for (int q = 0; q < 24; q++) {
        int dst[3];
        double Dr[3];
        for (int d = 0; d < 3; d++) {
            int v = src[rot.perm[q][d]];
            if (rot.sgn[q][d] < 0) v = (ng - 1) - v;
            dst[d] = v;
            Dr[d] = rot.sgn[q][d] * D[rot.perm[q][d]];
        }
        put(dst[0], dst[1], dst[2], Dr);
        double Di[3] = {-Dr[0], -Dr[1], -Dr[2]};
        put((ng - 1) - dst[0], (ng - 1) - dst[1], (ng - 1) - dst[2], Di);
    }
}

// erfcx(x) = exp(x^2) erfc(x) by Abramowitz & Stegun 7.1.26 (|error| ~ 1e-7),
// the approximation StePS/src/ewald_space.cc:537-561 uses for |arg| > 5.
__device__ double as_erfcx(double x)
{
    double sgn_term = 0.0;
    if (x < 0) {
        sgn_term = 2.0 * exp(x * x);
        x = -x;
        if (x == 0) return sgn_term - 1.0;
    } else if (x == 0) {
        return 1.0;
    }
    double v;
    if (x > 1e10) {
        v = 0.564189583547756286 / x;
    } else {
        double t = 1.0 / (1.0 + 0.3275911 * x);
        v = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))));
    }
    return sgn_term != 0.0 ? sgn_term - v : v;
}

// exp(+-k rho) erfc(k / (2 alpha) +- alpha rho) without overflow
// (StePS/src/ewald_space.cc:564-596).
__device__ double exp_erfc(double km, double rho, double alpha, bool plus)
{
    double a2 = km / (2.0 * alpha);
    double ar = alpha * rho;
    double arg = plus ? (a2 + ar) : (a2 - ar);
    double common = -(a2 * a2 + ar * ar);
    if (arg > 5.0) return exp(common) * as_erfcx(arg);
    if (arg < -5.0) return 2.0 * exp(-km * rho) - exp(common) * as_erfcx(-arg);
    return exp(plus ? km * rho : -km * rho) * erfc(arg);
}

// Nearest-image wrap of dz as StePS/src/ewald_space.cc:600-609 computes it.
__device__ double wrap_dz(double dz, double lz)
{
    double half = 0.5 * lz;
    if (dz > half) dz -= lz * floor((dz + half) / lz);
    if (dz <= -half) dz -= lz * floor((dz - half) / lz);
    return dz;
}

__global__ void k_s1r2_table(int nrho, int nz, double rho_max, double lz, double alpha, int nmax, int mmax,
                             double *__restrict__ tab)
{
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nrho * nz) return;
    int ir = id / nz, iz = id % nz;
    double drho = rho_max / (double)(nrho - 1 > 1 ? nrho - 1 : 1);
    double dzc = lz / (double)nz;
    double rho = (double)ir * drho;
    double z = ((double)iz + 0.5) * dzc - 0.5 * lz;
    // S1R2ewald_force_pair(dx = rho, dy = 0, dz = z): StePS/src/ewald_space.cc:618-752.
    double dx = rho, dy = 0.0, dz = wrap_dz(z, lz);
    double rho2 = dx * dx + dy * dy;
    double rr = sqrt(rho2);
    double Fxr = 0, Fzr = 0;
    // alpha = 0 with mmax = 0 is what the reference's PERIODIC_Z_RSPACELOOKUP
    // build passes (StePS/src/main.cc:650, :683): a direct real-space image sum
    // with no k-space part (StePS/src/ewald_space.cc:710-750), summed in its
    // order -- n = 0, then -n, +n for n = 1..nmax -- for the same rounding.
    const bool direct = alpha == 0.0 && mmax == 0;
    if (direct) {
        double r2 = rho2 + dz * dz;
        if (r2 >= 1e-18) {
            double r = sqrt(r2);
            double invr3 = 1.0 / (r2 * r);
            Fxr -= dx * invr3;
            Fzr -= dz * invr3;
        }
    }
    for (int n = direct ? 1 : -nmax; n <= nmax; ++n) {
        if (direct) {
            for (int sign = -1; sign <= 1; sign += 2) {
                double dzn = dz + (double)(sign * n) * lz;
                double r2 = rho2 + dzn * dzn;
                if (r2 < 1e-18) continue;
                double r = sqrt(r2);
                double invr3 = 1.0 / (r2 * r);
                Fxr -= dx * invr3;
                Fzr -= dzn * invr3;
            }
            continue;
        }
        double dzn = dz + (double)n * lz;
        double r2 = rho2 + dzn * dzn;
        if (r2 < 1e-18) continue;
        double r = sqrt(r2);
        double invr3 = 1.0 / (r2 * r);
        double ar = alpha * r;
        double co = (erfc(ar) + (2.0 / 1.7724538509055160272981674833411) * ar * exp(-ar * ar)) * invr3;
        Fxr -= dx * co;
        Fzr -= dzn * co;
    }
    double Frk = 0, Fzk = 0;
    double invL = 1.0 / lz;
    for (int m = 1; m <= mmax; ++m) {
        double km = (2.0 * PI * m) * invL;
        double tp = exp_erfc(km, rr, alpha, true);
        double tm = exp_erfc(km, rr, alpha, false);
        double B = tp + tm;
        double dB = km * (tp - tm);
        Frk += (2.0 * invL) * cos(km * dz) * dB;
        Fzk -= (2.0 * invL) * km * sin(km * dz) * B;
    }
    if (rr > 1e-12) Frk += -(2.0 * invL / rr) * (1.0 - exp(-alpha * alpha * rho2));
    double Fx = Fxr + (rr > 0 ? Frk * dx / rr : 0.0);
    double Fz = Fzr + Fzk;
    double zw = wrap_dz(z, lz);
    double r2 = rho * rho + zw * zw;
    double Frn = 0, Fzn = 0;
    if (r2 > 0) {
        double r = sqrt(r2);
        double i3 = 1.0 / (r * r * r);
        Frn = -rho * i3;
        Fzn = -zw * i3;
    }
    tab[2 * (size_t)id] = Fx - Frn;
    tab[2 * (size_t)id + 1] = Fz - Fzn;
}

// ---- cylindrical radial background multiplier (finite Ewald cylinder) ----
//
// RADIAL_FORCE_TABLE[i] for S1xR2 comoving runs: the radial pull of the matter
// outside the simulation cylinder relative to an infinite cylinder, at
// r_i = R i / (size - 1), by the trapezoid rule over `accuracy` intervals of
// Y in [0, R] (StePS/src/utils.cc:162-228). The integrand is the reference's
// closed form, evaluated with the same operation order (squares as products,
// square roots, no contraction); the trapezoid terms are summed per thread
// in order and the threads' sums in a fixed tree, so the table is
// deterministic and within rounding of the reference's sequential sum.
constexpr double RADIAL_PI = 3.14159265358979323846264338327950288419716939937510;
constexpr int RADIAL_THREADS = 128;

__device__ double radial_integrand(double R, double lz, double a, double Y, bool at_edge)
{
    const double s = sqrt(R * R - Y * Y);
    if (at_edge)  // a = R (utils.cc:186-191)
        return -2 * log((sqrt(lz * lz + 2 * (R * R) + 2 * R * s) + lz) / (sqrt(lz * lz + 2 * (R * R) - 2 * R * s) + lz));
    const double f1 = -2 * log((sqrt(lz * lz + R * R + a * a + 2 * a * s) + lz) / (sqrt(lz * lz + R * R + a * a - 2 * a * s) + lz));
    const double f2 = log((R * R + a * a + 2 * a * s) / (R * R + a * a - 2 * a * s));
    return f1 + f2;
}

__global__ void __launch_bounds__(RADIAL_THREADS) k_radial_table(double R, double lz, int size, int accuracy,
                                                                 double *__restrict__ out)
{
    __shared__ double part[RADIAL_THREADS];
    const int i = blockIdx.x + 1;  // entry 0 is interpolated afterwards
    const double step = R / (double)accuracy;
    double a = i == size - 1 ? R : R / (double)(size - 1) * i;
    const bool edge = a >= R;
    if (edge) a = R;
    // thread t sums the contiguous terms j in [j0, j1) in order
    const int per = (accuracy + RADIAL_THREADS - 1) / RADIAL_THREADS;
    const int j0 = 1 + threadIdx.x * per, j1 = min(accuracy + 1, j0 + per);
    double sum = 0.0;
    for (int j = j0; j < j1; j++) {
        const double ip = radial_integrand(R, lz, a, (j - 1) * step, edge);
        const double in = radial_integrand(R, lz, a, j * step, edge);
        sum += step * (ip + in) * 0.5;
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = RADIAL_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double total = part[0];
        out[i] = edge ? 2 * (total + RADIAL_PI * R) / (2 * RADIAL_PI * R) : 2 * total / (2 * RADIAL_PI * a);
    }
}

// Entry 0 by the reference's linear extrapolation from entries 1 and 2, taken
// at r = 2R/size and 4R/size (utils.cc:224-227, linear_interpolation utils.cc:24-37).
__global__ void k_radial_table0(double R, int size, double *out)
{
    if (size < 3) {
        out[0] = 0.0;
        return;
    }
    const double x1 = 2 * R / (double)size, x2 = 4 * R / (double)size;
    const double A = (out[2] - out[1]) / (x2 - x1);
    const double B = out[1] - A * x1;
    out[0] = A * 0.0 + B;
}

}  // namespace

}  // namespace steps

using namespace steps;

extern "C" {

int steps_gpu_build_radial_table(int size, double rsim, double lz, int accuracy)
{
    struct A {
        int size;
        double rsim, lz;
        int accuracy;
    } a{size, rsim, lz, accuracy};
    return run_guarded(
        [](void *p) {
            A &a = *static_cast<A *>(p);
            require_init();
            Ctx &c = ctx();
            if (a.size < 2 || a.size > (1 << 24) || a.accuracy < 1 || a.accuracy > (1 << 24) || !(a.rsim > 0) ||
                !(a.lz > 0))
                fail(STEPS_E_ARG, "build_radial_table: size >= 2, accuracy >= 1, rsim > 0 and lz > 0 required");
            double *tab = c.radial.ensure<double>(a.size);
            k_radial_table<<<a.size - 1, RADIAL_THREADS, 0, c.stream>>>(a.rsim, a.lz, a.size, a.accuracy, tab);
            note_launch("k_radial_table");
            k_radial_table0<<<1, 1, 0, c.stream>>>(a.rsim, a.size, tab);
            note_launch("k_radial_table0");
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
            c.radial_size = a.size;
        },
        &a);
}

int steps_gpu_get_radial_table(double *out)
{
    return run_guarded(
        [](void *p) {
            require_init();
            Ctx &c = ctx();
            if (!p) fail(STEPS_E_ARG, "out is NULL");
            if (c.radial_size <= 0) fail(STEPS_E_STATE, "no radial table");
            STEPS_CUDA(cudaMemcpyAsync(p, c.radial.as<double>(), sizeof(double) * c.radial_size,
                                       cudaMemcpyDeviceToHost, c.stream));
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
        },
        out);
}

int steps_gpu_build_table_t3(int ngrid, double L, double alpha, double rel_cut, double rec_cut, double real_radius,
                             double rec_radius)
{
    struct A {
        int ngrid;
        double L, alpha, rel_cut, rec_cut, real_radius, rec_radius;
    } a{ngrid, L, alpha, rel_cut, rec_cut, real_radius, rec_radius};
    return run_guarded(
        [](void *p) {
            A &a = *static_cast<A *>(p);
            require_init();
            Ctx &c = ctx();
            if (a.ngrid < 3 || a.ngrid > 1023 || (a.ngrid % 2) == 0)
                fail(STEPS_E_ARG, "build_table_t3: ngrid must be odd and in [3, 1023]");
            if (!(a.L > 0) || !(a.alpha > 0) || a.real_radius <= 0 || a.rec_radius <= 0 || a.real_radius > 40 ||
                a.rec_radius > 40)
                fail(STEPS_E_ARG, "build_table_t3: bad Ewald parameters");
            std::vector<int4> ri = lattice(a.real_radius), ki = lattice(a.rec_radius);
            DevBuf dri, dki;
            int4 *pri = dri.ensure<int4>(ri.size());
            int4 *pki = dki.ensure<int4>(ki.size());
            STEPS_CUDA(cudaMemcpyAsync(pri, ri.data(), ri.size() * sizeof(int4), cudaMemcpyHostToDevice, c.stream));
            STEPS_CUDA(cudaMemcpyAsync(pki, ki.data(), ki.size() * sizeof(int4), cudaMemcpyHostToDevice, c.stream));
            size_t cnt = 3 * (size_t)a.ngrid * a.ngrid * a.ngrid;
            double *tab = c.t3.ensure<double>(cnt);
            STEPS_CUDA(cudaMemsetAsync(tab, 0, cnt * sizeof(double), c.stream));
            int span = a.ngrid - a.ngrid / 2;
            long long total = (long long)span * span * span;
            k_t3_table<<<(unsigned)div_up((int)total, 128), 128, 0, c.stream>>>(
                a.ngrid, a.L, a.alpha, pri, (int)ri.size(), pki, (int)ki.size(), a.rel_cut, a.rec_cut,
                cube_rotations(), tab);
            note_launch("k_t3_table");
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
            dri.release();
            dki.release();
            c.t3_ng = a.ngrid;
            c.t3_version++;
        },
        &a);
}

int steps_gpu_build_table_s1r2(int nrho, int nz, double rho_max, double lz, double alpha, int nmax, int mmax)
{
    struct A {
        int nrho, nz;
        double rho_max, lz, alpha;
        int nmax, mmax;
    } a{nrho, nz, rho_max, lz, alpha, nmax, mmax};
    return run_guarded(
        [](void *p) {
            A &a = *static_cast<A *>(p);
            require_init();
            Ctx &c = ctx();
            if (a.nrho < 1 || a.nz < 1 || (long long)a.nrho * a.nz > (1LL << 28))
                fail(STEPS_E_ARG, "build_table_s1r2: bad shape");
            // alpha = 0 with mmax = 0: direct real-space sums, up to the 1e5 images
            // per side of the reference's IS_PERIODIC >= 4 setting (StePS/src/main.cc:624).
            const bool direct = a.alpha == 0.0 && a.mmax == 0;
            if (!(a.lz > 0) || !(direct || a.alpha > 0) || !(a.rho_max >= 0) || a.nmax < 0 || a.mmax < 0 ||
                a.nmax > (direct ? 100000 : 10000) || a.mmax > 10000)
                fail(STEPS_E_ARG, "build_table_s1r2: bad Ewald parameters");
            size_t cnt = 2 * (size_t)a.nrho * a.nz;
            double *tab = c.s1r2.ensure<double>(cnt);
            k_s1r2_table<<<div_up(a.nrho * a.nz, 128), 128, 0, c.stream>>>(a.nrho, a.nz, a.rho_max, a.lz, a.alpha,
                                                                         a.nmax, a.mmax, tab);
            note_launch("k_s1r2_table");
            STEPS_CUDA(cudaStreamSynchronize(c.stream));
            c.nrho = a.nrho;
            c.nz = a.nz;
            c.s1r2_version++;
        },
        &a);
}

}  // extern "C"
