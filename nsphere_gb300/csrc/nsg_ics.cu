// nsg_ics.cu -- seeded initial conditions generated on the GPU, in G = M = a = 1
// units, straight into the resident state (no host arrays, no upload):
//   * Plummer: inverse-CDF radii r = (u^(-2/3) - 1)^(-1/2) and the Aarseth, Henon &
//     Wielen (1974) rejection for q = v / v_esc, g(q) = q^2 (1 - q^2)^(7/2) < 0.1;
//   * Hernquist (1990), truncated at r_max: inverse-CDF radii of M(r) = r^2/(1+r)^2
//     and speeds from the isotropic distribution function f(E) by rejection under a
//     bound found per particle (grid search and golden-section refinement), or from
//     the Osipkov-Merritt f(Q) with anisotropy radius r_a (below).
// Directions use the reference's mapping v_r = v mu, ell = r v sqrt(1 - mu^2), mu
// uniform in [-1, 1] (nsphere.c:4805-4808, 4914).  The state is then sorted by
// radius and the ids are set to the radial rank, as the reference remaps them
// (nsphere.c:4908-4920).
//
// Random numbers come from a counter-based generator: draw j of particle i is a
// SplitMix64 finaliser (Steele, Lea & Flood 2014) applied twice to (seed, i, j), so a
// particle's draws do not depend on the launch shape or on other particles'
// rejections: draw 0 is the radius, draw 1 the direction, draws 2 + 2a and 3 + 2a the
// a-th rejection attempt.  nsphere_gb300/ics.py restates the generators with the same
// draws for the tests; this file is compiled without multiply-add contraction so that
// every operation rounds as numpy's does.
#include <cmath>
#include <vector>

#include "nsg_internal.cuh"

namespace nsg {

constexpr int kIcMaxAttempts = 1 << 16;

__host__ __device__ __forceinline__ uint64_t ic_mix(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Uniform double in [0, 1) with 53 random bits.
__host__ __device__ __forceinline__ double ic_uniform(uint64_t seed, uint64_t i, uint64_t j)
{
    const uint64_t h = ic_mix(ic_mix(seed ^ (i * 0xD1B54A32D192ED03ull)) + j);
    return (double)(h >> 11) * 0x1p-53;
}

// Isotropic Hernquist f(E) for binding energy eps in (0, 1), G = M = a = 1
// (Hernquist 1990, eq. 17), without the constant 1/(8 sqrt(2) pi^3).
__host__ __device__ __forceinline__ double hq_df(double eps)
{
    const double lim = 1.0 - 1e-15;
    const double e = eps < 0.0 ? 0.0 : (eps > lim ? lim : eps);
    const double q = sqrt(e), q2 = q * q;
    const double val = 3.0 * asin(q) + q * sqrt(1.0 - q2) * (1.0 - 2.0 * q2) * (8.0 * q2 * q2 - 8.0 * q2 - 3.0);
    const double w = 1.0 - q2;
    return val / (w * w * sqrt(w));
}

__global__ void k_ic_plummer(uint64_t seed, int64_t n, double *r_out, double *v_out, double *l_out,
                             int32_t *id_out, double *mu_out, unsigned int *status)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double u = 1e-10 + (1.0 - 1e-10) * ic_uniform(seed, i, 0);
        const double r = 1.0 / sqrt(pow(u, -2.0 / 3.0) - 1.0);
        double q = 0.0;
        int a = 0;
        for (; a < kIcMaxAttempts; a++) {
            const double x1 = ic_uniform(seed, i, 2 + 2 * (uint64_t)a);
            const double x2 = ic_uniform(seed, i, 3 + 2 * (uint64_t)a);
            const double w = 1.0 - x1 * x1;
            if (0.1 * x2 < x1 * x1 * (w * w * w * sqrt(w))) { q = x1; break; }
        }
        if (a == kIcMaxAttempts) atomicOr(status, NSG_ST_IC_REJECT);
        const double v = q * sqrt(2.0) / sqrt(sqrt(1.0 + r * r));
        const double mu = 2.0 * ic_uniform(seed, i, 1) - 1.0;
        r_out[i] = r;
        v_out[i] = v * mu;
        l_out[i] = r * v * sqrt(fmax(0.0, 1.0 - mu * mu));
        id_out[i] = (int32_t)i;
        if (mu_out) mu_out[i] = mu;
    }
}

// Bound of the rejection target g(x) = x^2 f(psi (1 - x^2)) on [0, 1] at one psi:
// the best of 64 points x_j = (j/64)^2 (dense near 0, where the peak moves as psi -> 1),
// refined by 40 golden-section steps around it, times 1.3.
__host__ __device__ __forceinline__ double hq_target(double psi, double x)
{
    return x * x * hq_df(psi * (1.0 - x * x));
}

__host__ __device__ __forceinline__ double hq_bound(double psi)
{
    int jb = 1;
    double gb = -1.0;
    for (int j = 1; j <= 64; j++) {
        const double t = j / 64.0;
        const double g = hq_target(psi, t * t);
        if (g > gb) { gb = g; jb = j; }
    }
    const double tl = (jb - 1) / 64.0, th = (jb < 64 ? jb + 1 : 64) / 64.0;
    double a = tl * tl, b = th * th;
    const double ig = 0.6180339887498949;           // (sqrt(5) - 1) / 2
    double c = b - ig * (b - a), d = a + ig * (b - a);
    double gc = hq_target(psi, c), gd = hq_target(psi, d);
    for (int it = 0; it < 40; it++) {
        if (gc > gd) { b = d; d = c; gd = gc; c = b - ig * (b - a); gc = hq_target(psi, c); }
        else { a = c; c = d; gc = gd; d = a + ig * (b - a); gd = hq_target(psi, d); }
    }
    const double m = fmax(gb, fmax(gc, gd));
    return m * 1.3 + 1e-300;
}

__global__ void k_ic_hernquist(uint64_t seed, int64_t n, double umax, double *r_out, double *v_out,
                               double *l_out, int32_t *id_out, double *mu_out, unsigned int *status)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double s = sqrt(umax * ic_uniform(seed, i, 0));
        const double r = fmax(s / (1.0 - s), 1e-12);
        const double psi = 1.0 / (1.0 + r);
        const double bound = hq_bound(psi);
        double x = 0.0;
        int a = 0;
        for (; a < kIcMaxAttempts; a++) {
            const double xx = ic_uniform(seed, i, 2 + 2 * (uint64_t)a);
            const double yy = ic_uniform(seed, i, 3 + 2 * (uint64_t)a) * bound;
            if (yy < hq_target(psi, xx)) { x = xx; break; }
        }
        if (a == kIcMaxAttempts) atomicOr(status, NSG_ST_IC_REJECT);
        const double w = x * sqrt(2.0 * psi);
        const double mu = 2.0 * ic_uniform(seed, i, 1) - 1.0;
        r_out[i] = r;
        v_out[i] = w * mu;
        l_out[i] = r * w * sqrt(fmax(0.0, 1.0 - mu * mu));
        id_out[i] = (int32_t)i;
        if (mu_out) mu_out[i] = mu;
    }
}

// Osipkov-Merritt anisotropy (Osipkov 1979; Merritt 1985) on the Hernquist halo: the
// distribution function depends on Q = E + L^2/(2 r_a^2) through the Eddington
// inversion of rho_Q = (1 + r^2/r_a^2) rho.  For Hernquist the added density
// r^2 rho / r_a^2 = (Psi^2 - Psi^3) / (2 pi r_a^2) inverts in closed form, so in the
// units of hq_df
//   f(Q) = hq_df(Q) + (8 / r_a^2) sqrt(Q) (1 - 2Q),  clamped at 0.
// At fixed r, w = (v_r, v_t sqrt(1 + r^2/r_a^2)) is then isotropic with speed density
// w^2 f(Psi - w^2/2): the isotropic sampler draws it, and v_t = w_t / sqrt(1 + r^2/r_a^2).
__host__ __device__ __forceinline__ double om_target(double psi, double x, double k)
{
    const double q = psi * (1.0 - x * x);
    const double f = hq_df(q) + k * sqrt(q) * (1.0 - 2.0 * q);
    return x * x * (f > 0.0 ? f : 0.0);
}

__host__ __device__ __forceinline__ double om_bound(double psi, double k)
{
    int jb = 1;
    double gb = -1.0;
    for (int j = 1; j <= 64; j++) {
        const double t = j / 64.0;
        const double g = om_target(psi, t * t, k);
        if (g > gb) { gb = g; jb = j; }
    }
    const double tl = (jb - 1) / 64.0, th = (jb < 64 ? jb + 1 : 64) / 64.0;
    double a = tl * tl, b = th * th;
    const double ig = 0.6180339887498949;
    double c = b - ig * (b - a), d = a + ig * (b - a);
    double gc = om_target(psi, c, k), gd = om_target(psi, d, k);
    for (int it = 0; it < 40; it++) {
        if (gc > gd) { b = d; d = c; gd = gc; c = b - ig * (b - a); gc = om_target(psi, c, k); }
        else { a = c; c = d; gc = gd; d = a + ig * (b - a); gd = om_target(psi, d, k); }
    }
    const double m = fmax(gb, fmax(gc, gd));
    return m * 1.3 + 1e-300;
}

__global__ void k_ic_hernquist_om(uint64_t seed, int64_t n, double umax, double r_a, double *r_out,
                                  double *v_out, double *l_out, int32_t *id_out, double *mu_out,
                                  unsigned int *status)
{
    const double k = 8.0 / (r_a * r_a);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double s = sqrt(umax * ic_uniform(seed, i, 0));
        const double r = fmax(s / (1.0 - s), 1e-12);
        const double psi = 1.0 / (1.0 + r);
        const double bound = om_bound(psi, k);
        double x = 0.0;
        int a = 0;
        for (; a < kIcMaxAttempts; a++) {
            const double xx = ic_uniform(seed, i, 2 + 2 * (uint64_t)a);
            const double yy = ic_uniform(seed, i, 3 + 2 * (uint64_t)a) * bound;
            if (yy < om_target(psi, xx, k)) { x = xx; break; }
        }
        if (a == kIcMaxAttempts) atomicOr(status, NSG_ST_IC_REJECT);
        const double w = x * sqrt(2.0 * psi);
        const double mu = 2.0 * ic_uniform(seed, i, 1) - 1.0;
        const double wr = w * mu, wt = w * sqrt(fmax(0.0, 1.0 - mu * mu));
        const double ra = r / r_a;
        const double vt = wt / sqrt(1.0 + ra * ra);
        r_out[i] = r;
        v_out[i] = wr;
        l_out[i] = r * vt;
        id_out[i] = (int32_t)i;
        if (mu_out) mu_out[i] = mu;
    }
}

__global__ void k_ic_rank_ids(int32_t *id, int64_t n)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        id[k] = (int32_t)k;
}

}  // namespace nsg

using namespace nsg;

static int generate(nsg_ctx *c, int model, int64_t n, uint64_t seed, double r_max, double r_a)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (model != NSG_IC_PLUMMER && model != NSG_IC_HERNQUIST) return set_err(c, NSG_EINVAL, "unknown model");
    if (model == NSG_IC_HERNQUIST && !(r_max > 0.0 && std::isfinite(r_max)))
        return set_err(c, NSG_EINVAL, "r_max must be positive and finite");
    if (!(r_a > 0.0)) return set_err(c, NSG_EINVAL, "r_a must be positive");
    if (int rc = begin_upload(c, n)) return rc;
    cudaStream_t s = c->stream;
    double *mu = c->p.carry_aux ? c->aux[0] : nullptr;
    cudaError_t e = cudaMemsetAsync(&c->ctr->status, 0, 4, s);
    if (e != cudaSuccess) return cuda_err(c, e, "generate");
    if (model == NSG_IC_PLUMMER) {
        k_ic_plummer<<<grid_for(c, n, 256), 256, 0, s>>>(seed, n, c->r[0], c->vr[0], c->ell[0], c->id[0], mu,
                                                         &c->ctr->status);
    } else if (std::isinf(r_a)) {
        const double umax = (r_max / (1.0 + r_max)) * (r_max / (1.0 + r_max));
        k_ic_hernquist<<<grid_for(c, n, 256), 256, 0, s>>>(seed, n, umax, c->r[0], c->vr[0], c->ell[0], c->id[0],
                                                           mu, &c->ctr->status);
    } else {
        const double umax = (r_max / (1.0 + r_max)) * (r_max / (1.0 + r_max));
        k_ic_hernquist_om<<<grid_for(c, n, 256), 256, 0, s>>>(seed, n, umax, r_a, c->r[0], c->vr[0], c->ell[0],
                                                              c->id[0], mu, &c->ctr->status);
    }
    c->launches += 1;
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, "generate");
    // radial order, then ids = radial rank
    if (int rc = sort_state(c)) return rc;
    k_ic_rank_ids<<<grid_for(c, n, 256), 256, 0, s>>>(c->id[c->cur], n);
    c->inv_valid = false;
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, "generate");
    return NSG_OK;
}

extern "C" int nsg_generate(nsg_ctx *c, int model, int64_t n, uint64_t seed, double r_max)
{
    return generate(c, model, n, seed, r_max, INFINITY);
}

extern "C" int nsg_generate_om(nsg_ctx *c, int64_t n, uint64_t seed, double r_max, double r_a)
{
    if (c && !(r_a > 0.0 && std::isfinite(r_a))) return set_err(c, NSG_EINVAL, "r_a must be positive and finite");
    return generate(c, NSG_IC_HERNQUIST, n, seed, r_max, r_a);
}
