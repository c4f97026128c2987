// loader.cpp -- seeded particle load for the device-resident simulation: OSIRIS lattice
// positions, charge from the density profile, thermal + fluid momenta.
//
//   lattice / charge    source/spec/psource/os-psource-std.f03:759-1120 (positions :845-870,
//                       charge sign(1/ppc, rqm) * den :837,915; cells visited with x slowest)
//   momenta             source/spec/os-spec-udist.f03:452-850 (uth * gaussian per component,
//                       then the relativistic ufl boost :716-748)
//   Mersenne Twister    source/random/os-random-mt.f03:84-149 (seed word 0 = seed ^ 0x80000000,
//                       first draw = tempered last initialisation word)
//   gaussian            source/random/os-random-class.f03:348-392 (polar Box-Muller)
//
// Compiled with -ffp-contract=off: the same roundings on x86_64 and aarch64, so a load is
// bit-identical wherever it runs.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/osiris_gb300.h"

namespace {

struct Rng {
    uint32_t mt[624];
    int next;
    int have_gauss;
    double gauss;
};
static_assert(sizeof(Rng) <= OSG_RNG_BYTES, "OSG_RNG_BYTES too small");

void rng_seed(Rng &r, int seed)
{
    r.mt[0] = (uint32_t)seed ^ 0x80000000u;
    for (int i = 1; i < 624; i++)
        r.mt[i] = 1812433253u * (r.mt[i - 1] ^ (r.mt[i - 1] >> 30)) + (uint32_t)i;
    r.next = 623;
    r.have_gauss = 0;
    r.gauss = 0.0;
}

void rng_refill(Rng &r)
{
    const uint32_t A = 0x9908b0dfu;
    for (int k = 0; k < 624; k++) {
        const uint32_t y = (r.mt[k] & 0x80000000u) | (r.mt[(k + 1) % 624] & 0x7fffffffu);
        r.mt[k] = r.mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
    }
    r.next = 0;
}

int32_t rng_int32(Rng &r)
{
    if (r.next >= 624) rng_refill(r);
    uint32_t y = r.mt[r.next++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return (int32_t)y;
}

double rng_gauss(Rng &r)
{
    if (r.have_gauss) {
        r.have_gauss = 0;
        return r.gauss;
    }
    double a, b, s;
    for (;;) {
        a = ((double)rng_int32(r) + 0.5) * (1.0 / 2147483648.0);
        b = ((double)rng_int32(r) + 0.5) * (1.0 / 2147483648.0);
        s = a * a + b * b;
        if (s < 1.0 && s > 0.0) break;
    }
    const double f = std::sqrt(-2.0 * std::log(s) / s);
    r.gauss = a * f;
    r.have_gauss = 1;
    return b * f;
}

template <typename T> T sqrt_t(T v) { return std::sqrt(v); }

template <typename T>
long load(Rng &rng, int dim, const int *nx, const int *ppc, const double *dx, double rqm,
          const double *uth, const double *ufl, double amp, double kmode, int *ix, T *x, T *u,
          T *q)
{
    int per_cell = 1;
    for (int d = 0; d < dim; d++) per_cell *= ppc[d];
    const T charge_unit = (T)(rqm < 0 ? -1.0 : 1.0) * ((T)1 / (T)per_cell);
    T offs[3][64];
    for (int d = 0; d < dim; d++) {
        const T half = (T)0.5 / (T)ppc[d];
        for (int i = 1; i <= ppc[d]; i++) offs[d][i - 1] = (T)(2 * i - 1 - ppc[d]) * half;
    }
    const int ny = dim > 1 ? nx[1] : 1, nz = dim > 2 ? nx[2] : 1;
    const int py = dim > 1 ? ppc[1] : 1, pz = dim > 2 ? ppc[2] : 1;
    const double L1 = nx[0] * dx[0];
    const double two_pi = 6.283185307179586476925286766559;
    long n = 0;
    for (int c1 = 1; c1 <= nx[0]; c1++)
        for (int c2 = 1; c2 <= ny; c2++)
            for (int c3 = 1; c3 <= nz; c3++)
                for (int a = 0; a < ppc[0]; a++)
                    for (int b = 0; b < py; b++)
                        for (int c = 0; c < pz; c++) {
                            const int cell[3] = {c1, c2, c3}, sub[3] = {a, b, c};
                            for (int d = 0; d < dim; d++) {
                                x[dim * n + d] = offs[d][sub[d]];
                                ix[dim * n + d] = cell[d];
                            }
                            const double xp = (c1 - 0.5 + (double)offs[0][a]) * dx[0];
                            const T den = (T)(1.0 + amp * std::cos(two_pi * kmode * xp / L1));
                            q[n] = den * charge_unit;
                            n++;
                        }
    const T f1 = (T)ufl[0], f2 = (T)ufl[1], f3 = (T)ufl[2];
    const T boost = (T)1 / (sqrt_t<T>((T)1 + f1 * f1 + f2 * f2 + f3 * f3) + (T)1);
    for (long p = 0; p < n; p++) {
        T *v = u + 3 * p;
        v[0] = (T)((T)uth[0] * rng_gauss(rng));
        v[1] = (T)((T)uth[1] * rng_gauss(rng));
        v[2] = (T)((T)uth[2] * rng_gauss(rng));
        const T g = sqrt_t<T>((T)1 + v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const T s = boost * (v[0] * f1 + v[1] * f2 + v[2] * f3) + g;
        v[0] = v[0] + s * f1;
        v[1] = v[1] + s * f2;
        v[2] = v[2] + s * f3;
    }
    return n;
}

} // namespace

extern "C" int osg_rng_seed(void *rng, int seed)
{
    if (!rng) return OSG_ERR_ARG;
    rng_seed(*static_cast<Rng *>(rng), seed);
    return OSG_OK;
}

extern "C" long osg_load_lattice(void *rng, int precision, int dim, const int *nx,
                                 const int *ppc, const double *dx, double rqm,
                                 const double *uth, const double *ufl, double amp, double kmode,
                                 int *ix, void *x, void *u, void *q)
{
    if (!rng || !nx || !ppc || !dx || !uth || !ufl || !ix || !x || !u || !q) return OSG_ERR_ARG;
    if (dim < 1 || dim > 3) return OSG_ERR_ARG;
    for (int d = 0; d < dim; d++)
        if (nx[d] < 1 || ppc[d] < 1 || ppc[d] > 64) return OSG_ERR_ARG;
    Rng &r = *static_cast<Rng *>(rng);
    if (precision == 32)
        return load<float>(r, dim, nx, ppc, dx, rqm, uth, ufl, amp, kmode, ix, (float *)x,
                           (float *)u, (float *)q);
    if (precision == 64)
        return load<double>(r, dim, nx, ppc, dx, rqm, uth, ufl, amp, kmode, ix, (double *)x,
                            (double *)u, (double *)q);
    return OSG_ERR_ARG;
}
