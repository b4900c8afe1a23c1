// Plain FP64 direct-summation kernels (all topologies): the GPU-side
// correctness reference, FP64 end to end.
//
// One thread per i particle, i in registers; j particles staged 128 at a time
// in shared memory as (x, y, z, m) double4 plus their softening, and visited
// in ascending j order, so each i's sum is taken in the order of the
// reference's sequential j loop (StePS/src/forces.cc:538). The j range may be
// split into chunks (blockIdx.y) whose FP64 partial sums are added in chunk
// order by the reduction, which also applies the background term.
#include "common.cuh"
#include "context.cuh"

namespace steps {

namespace {

constexpr int FP64_THREADS = 128;

enum Fp64Mode { M_R3 = 0, M_T3_EWALD, M_NEAREST3, M_S1_IMAGES, M_S1_NEAREST, M_S1_TABLE };

__device__ __forceinline__ int pos_mod(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

// Tensor-product T^3 table interpolation (StePS/src/ewald_space.cc:452-523,
// StePS/src/forces_cuda.cu:113-167): ORDER 2 = trilinear (2-point Lagrange),
// ORDER 4 = Catmull-Rom tricubic, on cell centres (i + 1/2) h - L/2.
template <int ORDER>
__device__ __forceinline__ void t3_interp_fp64(const double *__restrict__ tab, int ng, double L, double ih, double dx,
                                               double dy, double dz, double &Dx, double &Dy, double &Dz)
{
    double d[3] = {dx, dy, dz};
    int i0[3];
    double w[3][4];
    for (int k = 0; k < 3; k++) {
        double u = (d[k] + 0.5 * L) * ih - 0.5;
        double uf = floor(u);
        i0[k] = pos_mod((int)uf, ng);
        double t = u - uf;
        if (ORDER == 4) {
            double t2 = t * t, t3 = t2 * t;
            w[k][0] = -0.5 * t3 + t2 - 0.5 * t;
            w[k][1] = 1.5 * t3 - 2.5 * t2 + 1.0;
            w[k][2] = -1.5 * t3 + 2.0 * t2 + 0.5 * t;
            w[k][3] = 0.5 * t3 - 0.5 * t2;
        } else {
            w[k][0] = 1.0 - t;
            w[k][1] = t;
        }
    }
    constexpr int OFF = ORDER == 4 ? -1 : 0;
    double s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
    for (int a = 0; a < ORDER; a++) {
        int ix = pos_mod(i0[0] + OFF + a, ng);
        STEPS_CHECK_IDX(ix, ng, CK_T3_FP64);
#pragma unroll
        for (int b = 0; b < ORDER; b++) {
            int iy = pos_mod(i0[1] + OFF + b, ng);
            STEPS_CHECK_IDX(iy, ng, CK_T3_FP64);
            double wxy = w[0][a] * w[1][b];
            const double *row = tab + (size_t)(ix * ng + iy) * ng * 3;
#pragma unroll
            for (int c = 0; c < ORDER; c++) {
                int iz = pos_mod(i0[2] + OFF + c, ng);
                STEPS_CHECK_IDX(iz, ng, CK_T3_FP64);
                double ww = wxy * w[2][c];
                s0 += ww * __ldg(row + 3 * iz);
                s1 += ww * __ldg(row + 3 * iz + 1);
                s2 += ww * __ldg(row + 3 * iz + 2);
            }
        }
    }
    Dx = s0;
    Dy = s1;
    Dz = s2;
}

// (rho, z) table interpolation, NGP / CIC / TSC (StePS/src/ewald_space.cc:803-1048,
// StePS/src/forces_cuda.cu:188-455), then D_rho mapped to (x, y).
template <int ORDER>
__device__ __forceinline__ void s1r2_interp_fp64(const double *__restrict__ T, int nrho, int nz, double rho_max,
                                                 double lz, double dx, double dy, double dz, double &Dx, double &Dy,
                                                 double &Dz)
{
    double rho = sqrt(dx * dx + dy * dy);
    double half = 0.5 * lz;
    double drho = rho_max / (double)(nrho - 1 > 1 ? nrho - 1 : 1);
    double dzc = lz / (double)nz;
    double rr = rho < 0 ? 0 : (rho > rho_max ? rho_max : rho);
    double ur = drho > 0 ? rr / drho : 0.0;
    double uz = (dz + half) / dzc - 0.5;
    double Dr = 0, Dzz = 0;
    auto at = [&](int ir, int iz, int c) {
        STEPS_CHECK_IDX(ir, nrho, CK_S1_CELL);
        STEPS_CHECK_IDX(iz, nz, CK_S1_CELL);
        return __ldg(T + ((size_t)ir * nz + iz) * 2 + c);
    };
    if (ORDER == 0) {
        int ir = (int)floor(ur + 0.5);
        int iz = (int)floor(uz + 0.5);
        ir = ir < 0 ? 0 : (ir > nrho - 1 ? nrho - 1 : ir);
        iz = pos_mod(iz, nz);
        Dr = at(ir, iz, 0);
        Dzz = at(ir, iz, 1);
    } else if (ORDER == 2) {
        int ir0 = (int)floor(ur);
        double fr = ur - (double)ir0;
        if (ir0 < 0) { ir0 = 0; fr = 0; }
        if (ir0 > nrho - 2) { ir0 = nrho - 2 > 0 ? nrho - 2 : 0; fr = 1.0; }
        int ir1 = ir0 + 1;
        int iz0 = (int)floor(uz);
        double fz = uz - (double)iz0;
        iz0 = pos_mod(iz0, nz);
        int iz1 = pos_mod(iz0 + 1, nz);
        double w00 = (1.0 - fr) * (1.0 - fz), w10 = fr * (1.0 - fz), w01 = (1.0 - fr) * fz, w11 = fr * fz;
        Dr = w00 * at(ir0, iz0, 0) + w10 * at(ir1, iz0, 0) + w01 * at(ir0, iz1, 0) + w11 * at(ir1, iz1, 0);
        Dzz = w00 * at(ir0, iz0, 1) + w10 * at(ir1, iz0, 1) + w01 * at(ir0, iz1, 1) + w11 * at(ir1, iz1, 1);
    } else {
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
#pragma unroll
        for (int zr = 0; zr < 3; zr++) {
            double w0 = wr[0] * wz[zr], w1 = wr[1] * wz[zr], w2 = wr[2] * wz[zr];
            Dr += w0 * at(ir[0], izs[zr], 0) + w1 * at(ir[1], izs[zr], 0) + w2 * at(ir[2], izs[zr], 0);
            Dzz += w0 * at(ir[0], izs[zr], 1) + w1 * at(ir[1], izs[zr], 1) + w2 * at(ir[2], izs[zr], 1);
        }
    }
    double ex = rho > 0 ? dx / rho : 0.0;
    double ey = rho > 0 ? dy / rho : 0.0;
    Dx = Dr * ex;
    Dy = Dr * ey;
    Dz = Dzz;
}

__device__ __forceinline__ double nearest(double d, double L, double halfL)
{
    // Subtract L sign(d) once when |d| > L/2 (StePS/src/forces.cc:812-817).
    return fabs(d) > halfL ? d - copysign(L, d) : d;
}

template <int MODE, int ORDER>
__global__ void __launch_bounds__(FP64_THREADS)
    k_pair_fp64(const double4_16a *__restrict__ pj, const double *__restrict__ ej, int n, int id_min, int ni, int jchunk,
                KParams kp, Tables tb, double *__restrict__ part)
{
    __shared__ double4_16a sp[FP64_THREADS];
    __shared__ double se[FP64_THREADS];
    int t = threadIdx.x;
    int li = blockIdx.x * FP64_THREADS + t;
    bool active = li < ni;
    double4_16a pi = active ? pj[id_min + li] : make_double4_16a(0, 0, 0, 0);
    double ei = active ? ej[id_min + li] : 0.0;
    int j0 = blockIdx.y * jchunk;
    int j1 = min(n, j0 + jchunk);
    double ax = 0, ay = 0, az = 0;
    const double L = kp.L, halfL = kp.halfL;
    const double ih = MODE == M_T3_EWALD ? (double)tb.t3_ng / L : 0.0;
    for (int jb = j0; jb < j1; jb += FP64_THREADS) {
        int cnt = min(FP64_THREADS, j1 - jb);
        __syncthreads();
        if (t < cnt) {
            sp[t] = pj[jb + t];
            se[t] = ej[jb + t];
        }
        __syncthreads();
        for (int jj = 0; jj < cnt; ++jj) {
            double4_16a q = sp[jj];
            double b = ei + se[jj];
            double dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
            if (MODE == M_R3) {
                double r2 = dx * dx + dy * dy + dz * dz;
                double w = q.w * softening_fp64(r2, b);
                ax = fma(w, dx, ax);
                ay = fma(w, dy, ay);
                az = fma(w, dz, az);
            } else if (MODE == M_T3_EWALD || MODE == M_NEAREST3) {
                dx = nearest(dx, L, halfL);
                dy = nearest(dy, L, halfL);
                dz = nearest(dz, L, halfL);
                double r2 = dx * dx + dy * dy + dz * dz;
                double w = softening_fp64(r2, b);
                if (MODE == M_T3_EWALD) {
                    double Dx, Dy, Dz;
                    t3_interp_fp64<ORDER>(tb.t3, tb.t3_ng, L, ih, dx, dy, dz, Dx, Dy, Dz);
                    ax += q.w * (w * dx - Dx);
                    ay += q.w * (w * dy - Dy);
                    az += q.w * (w * dz - Dz);
                } else {
                    w *= q.w;
                    ax = fma(w, dx, ax);
                    ay = fma(w, dy, ay);
                    az = fma(w, dz, az);
                }
            } else if (MODE == M_S1_IMAGES) {
                // Images m in [-emax, emax] along z with |dz + mL| <= cutL
                // (StePS/src/forces.cc:1250-1290): per-j image sum, then added.
                double rho2 = dx * dx + dy * dy;
                double fx = 0, fy = 0, fz = 0;
                for (int m = -kp.emax; m <= kp.emax; ++m) {
                    double dzm = dz + (double)m * L;
                    if (fabs(dzm) <= kp.cutL) {
                        double w = q.w * softening_fp64(rho2 + dzm * dzm, b);
                        fx += w * dx;
                        fy += w * dy;
                        fz += w * dzm;
                    }
                }
                ax += fx;
                ay += fy;
                az += fz;
            } else if (MODE == M_S1_NEAREST) {
                dz = nearest(dz, L, halfL);
                double w = q.w * softening_fp64(dx * dx + dy * dy + dz * dz, b);
                ax = fma(w, dx, ax);
                ay = fma(w, dy, ay);
                az = fma(w, dz, az);
            } else {  // M_S1_TABLE
                dz = nearest(dz, L, halfL);
                double w = softening_fp64(dx * dx + dy * dy + dz * dz, b);
                double Dx, Dy, Dz;
                s1r2_interp_fp64<ORDER>(tb.s1r2, tb.nrho, tb.nz, tb.rho_max, L, dx, dy, dz, Dx, Dy, Dz);
                ax += q.w * (w * dx - Dx);
                ay += q.w * (w * dy - Dy);
                az += q.w * (w * dz - Dz);
            }
        }
    }
    if (active) {
        double *o = part + ((size_t)blockIdx.y * ni + li) * 3;
        o[0] = ax;
        o[1] = ay;
        o[2] = az;
    }
}

__global__ void k_pack64(const double *__restrict__ x, const double *__restrict__ m, int n, double4_16a *__restrict__ out)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_double4_16a(x[3 * (size_t)i], x[3 * (size_t)i + 1], x[3 * (size_t)i + 2], m[i]);
}

}  // namespace

namespace {

__global__ void k_reduce_fp64(const double *__restrict__ part, int S, int ni, int id_min, const double *__restrict__ x,
                              Background bg, double *__restrict__ F)
{
    int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= ni) return;
    double f[3] = {0, 0, 0};
    for (int s = 0; s < S; s++)
        for (int k = 0; k < 3; k++) f[k] += part[((size_t)s * ni + li) * 3 + k];
    add_background(bg, x + 3 * (size_t)(id_min + li), f);
    for (int k = 0; k < 3; k++) F[3 * (size_t)li + k] = f[k];
}

template <int MODE, int ORDER>
void launch_fp64(dim3 grid, int n, int id_min, int ni, int jchunk, const KParams &kp, const Tables &tb, double *part,
                 cudaStream_t st)
{
    Ctx &c = ctx();
    k_pair_fp64<MODE, ORDER><<<grid, FP64_THREADS, 0, st>>>(c.pack64.as<double4_16a>(), c.eps64.as<double>(), n, id_min, ni,
                                                            jchunk, kp, tb, part);
    note_launch("k_pair_fp64");
}

}  // namespace

Background background_of(const KParams &kp, const Tables &tb)
{
    Background bg{0, 0.0, kp.rsim, tb.radial, tb.radial_size};
    if (kp.comoving_bg == 0) return bg;
    if (kp.topology == STEPS_R3) {
        bg.mode = 1;
        bg.coef = kp.bg_coef;
    } else if (kp.topology == STEPS_S1R2) {
        bool table_mode = kp.is_periodic >= 2 && !kp.s1r2_images;
        if (kp.comoving_bg == 1 && !table_mode) {
            if (!tb.radial || tb.radial_size < 2) fail(STEPS_E_STATE, "S1R2 comoving run needs the radial force table");
            bg.mode = 3;
        } else {
            bg.mode = 2;
        }
        bg.coef = kp.bg_coef;
    }
    return bg;
}

void forces_fp64(const KParams &kp, const Tables &tb, const double *x, int n, int id_min, int ni, double *F)
{
    Ctx &c = ctx();
    cudaStream_t st = c.stream;
    c.pack64.ensure<double4_16a>(n);
    STEPS_CUDA(cudaEventRecord(c.phase[0], st));
    k_pack64<<<div_up(n, 256), 256, 0, st>>>(x, c.m64.as<double>(), n, c.pack64.as<double4_16a>());
    note_launch("k_pack64");
    STEPS_CUDA(cudaEventRecord(c.phase[1], st));

    // Enough blocks for several waves of the GPU: split the j range.
    int bx = div_up(ni, FP64_THREADS);
    int target = c.nsm * 16;
    int S = div_up(target, bx);
    int maxS = div_up(n, FP64_THREADS);
    if (S > maxS) S = maxS;
    if (S < 1) S = 1;
    int jchunk = div_up(div_up(n, S), FP64_THREADS) * FP64_THREADS;
    S = div_up(n, jchunk);
    double *part = c.partial.ensure<double>((size_t)S * ni * 3);
    dim3 grid(bx, S);

    if (kp.topology == STEPS_R3) {
        launch_fp64<M_R3, 0>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
    } else if (kp.topology == STEPS_T3) {
        if (kp.is_periodic >= 2) {
            if (kp.order == 4) launch_fp64<M_T3_EWALD, 4>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
            else launch_fp64<M_T3_EWALD, 2>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
        } else {
            launch_fp64<M_NEAREST3, 0>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
        }
    } else {
        if (kp.is_periodic < 2) launch_fp64<M_S1_NEAREST, 0>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
        else if (kp.s1r2_images) launch_fp64<M_S1_IMAGES, 0>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
        else if (kp.order == 0) launch_fp64<M_S1_TABLE, 0>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
        else if (kp.order == 2) launch_fp64<M_S1_TABLE, 2>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
        else launch_fp64<M_S1_TABLE, 4>(grid, n, id_min, ni, jchunk, kp, tb, part, st);
    }
    STEPS_CUDA(cudaEventRecord(c.phase[2], st));
    k_reduce_fp64<<<div_up(ni, 256), 256, 0, st>>>(part, S, ni, id_min, x, background_of(kp, tb), F);
    note_launch("k_reduce_fp64");
    STEPS_CUDA(cudaEventRecord(c.phase[3], st));
    c.phase_valid = true;
    c.last_pairs = (double)ni * (double)n;
}

}  // namespace steps
