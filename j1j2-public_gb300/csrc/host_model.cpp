// Host-side model helpers of libj1j2cuda (no GPU needed): the reference's KISS05 generator, the
// correlated random field of make_corr_rand_3d with an own radix-2 FFT, vacancies, KISS-seeded
// starts and the temperature ladder.  FP64 throughout; compiled without floating-point
// contraction so every expression rounds as written.
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

#include "../../include/j1j2c.h"

namespace {

// KISS05 (J:3614-3695): LCG + xorshift + two multiply-with-carry generators; INTEGER(4) wraps and
// ishft(.., -k) is a logical shift, so uint32 arithmetic restates it.
struct Kiss {
    uint32_t x = 0, y = 0, z = 0, w = 0;

    double next()
    {
        x = 69069u * x + 1327217885u;
        y ^= y << 13;
        y ^= y >> 17;
        y ^= y << 5;
        z = 18000u * (z & 65535u) + (z >> 16);
        w = 30903u * (w & 65535u) + (w >> 16);
        const uint32_t k = (x + y + (z << 16) + w) >> 1;
        return (double)k * 4.656612873077392578e-10;
    }

    // kissinit: seed shuffled by a 32-bit LCG, then four Park-Miller steps (Schrage)
    void seed(int32_t iinit)
    {
        int32_t idum = (int32_t)((uint32_t)iinit * 1099087573u);
        if (idum < 0 && idum != INT32_MIN) idum = -idum;
        if (idum == 0) idum = 1;
        if (idum >= 2147483647) idum = 2147483646;
        uint32_t* st[4] = {&x, &y, &z, &w};
        for (auto* v : st) {
            const int32_t k = idum / 127773;
            int64_t t = (int64_t)16807 * (idum - k * 127773) - (int64_t)2836 * k;
            idum = (int32_t)t;
            if (idum < 0) idum += 2147483647;
            *v = (uint32_t)(idum < 1 ? idum + 1 : idum);
        }
        (void)next();
    }
};

// gkiss05 (CR:48-76): polar method, second deviate cached
struct Gauss {
    Kiss k;
    double gset = 0.0;
    bool have = false;

    double next()
    {
        if (have) {
            have = false;
            return gset;
        }
        double v1, v2, s;
        do {
            v1 = 2.0 * k.next() - 1.0;
            v2 = 2.0 * k.next() - 1.0;
            s = v1 * v1 + v2 * v2;
        } while (!(s < 1.0 && s > 0.0));
        const double fac = std::sqrt(-2.0 * std::log(s) / s);
        gset = v1 * fac;
        have = true;
        return v2 * fac;
    }
};

// erfcc (CR:31-43): Chebyshev approximation of erfc
double erfcc(double x)
{
    const double z = std::fabs(x);
    const double t = 1.0 / (1.0 + 0.5 * z);
    const double poly =
        t * (1.00002368 +
             t * (.37409196 +
                  t * (.09678418 +
                       t * (-.18628806 +
                            t * (.27886807 +
                                 t * (-1.13520398 +
                                      t * (1.48851587 + t * (-.82215223 + t * .17087277))))))));
    double r = t * std::exp(((-z * z) - 1.26551223) + poly);
    if (x < 0.0) r = 2.0 - r;
    return r;
}

int nextpow2(int n)
{
    int p = 1;
    while (p < n) p *= 2;
    return p;
}

using cplx = std::complex<double>;

// In-place iterative radix-2 FFT of n points spaced by `stride`; sign -1 forward, +1 inverse
// (unscaled).
void fft1(cplx* a, int n, long stride, int sign, const std::vector<cplx>& tw)
{
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[(long)i * stride], a[(long)j * stride]);
    }
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len)
            for (int k = 0; k < half; ++k) {
                cplx w = tw[(size_t)k * step];
                if (sign > 0) w = std::conj(w);
                const cplx u = a[(long)(i + k) * stride];
                const cplx v = a[(long)(i + k + half) * stride] * w;
                a[(long)(i + k) * stride] = u + v;
                a[(long)(i + k + half) * stride] = u - v;
            }
    }
}

std::vector<cplx> twiddles(int n)
{
    std::vector<cplx> tw((size_t)(n / 2 > 0 ? n / 2 : 1));
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < n / 2; ++k)
        tw[k] = cplx(std::cos(2.0 * pi * k / n), -std::sin(2.0 * pi * k / n));
    return tw;
}

// 3D FFT of a[k][j][i] (dims f3, f2, f1; i fastest)
void fft3(std::vector<cplx>& a, int f1, int f2, int f3, int sign)
{
    const auto t1 = twiddles(f1), t2 = twiddles(f2), t3 = twiddles(f3);
    for (int k = 0; k < f3; ++k)
        for (int j = 0; j < f2; ++j) fft1(&a[((size_t)k * f2 + j) * f1], f1, 1, sign, t1);
    for (int k = 0; k < f3; ++k)
        for (int i = 0; i < f1; ++i) fft1(&a[(size_t)k * f2 * f1 + i], f2, f1, sign, t2);
    for (int j = 0; j < f2; ++j)
        for (int i = 0; i < f1; ++i) fft1(&a[(size_t)j * f1 + i], f3, (long)f1 * f2, sign, t3);
}

}  // namespace

namespace j1j2 {
// gkiss05 white noise after gkissinit(seed), n deviates in the reference's order (CR:256, 280-287)
void gauss_fill(int32_t seed, size_t n, double* out)
{
    Gauss gs;
    gs.k.seed(seed);
    for (size_t t = 0; t < n; ++t) out[t] = gs.next();
}

// the uniform map of CR:333-341 (x -> (2 (1 - erfcc(x / sqrt 2) / 2) - 1) * max_value)
double uniform_map(double v, double max_value)
{
    return (2.0 * (1.0 - 0.5 * erfcc(v / std::sqrt(2.0))) - 1.0) * max_value;
}
}  // namespace j1j2

extern "C" {

int j1j2c_corr_rand_3d(int32_t n1, int32_t n2, int32_t n3, double xi, int32_t seed,
                       int32_t do_uniform, double max_value, double* out)
{
    if (n1 < 1 || n2 < 1 || n3 < 1 || !out) return J1J2C_EINVAL;
    const int f1 = nextpow2(n1), f2 = nextpow2(n2), f3 = nextpow2(n3);
    const size_t nt = (size_t)f1 * f2 * f3;
    if (nt > (size_t)1 << 27) return J1J2C_EINVAL;
    std::vector<cplx> c(nt), x(nt);
    // C(dx,dy,dz) = exp(-r/xi), periodic distance on the padded cube (CR:261-268, CR:362-384)
    for (int k = 0; k < f3; ++k)
        for (int j = 0; j < f2; ++j)
            for (int i = 0; i < f1; ++i) {
                const int dx = i < f1 - i ? i : f1 - i, dy = j < f2 - j ? j : f2 - j,
                          dz = k < f3 - k ? k : f3 - k;
                const double r = std::sqrt((double)(dx * dx + dy * dy + dz * dz));
                double v;
                if (xi <= 0.0)
                    v = (r == 0.0) ? 1.0 : 0.0;
                else
                    v = std::exp(-r / xi);
                c[((size_t)k * f2 + j) * f1 + i] = cplx(v, 0.0);
            }
    // white noise in Fortran order after gkissinit(seed) (CR:256, CR:280-287)
    Gauss gs;
    gs.k.seed(seed);
    for (size_t t = 0; t < nt; ++t) x[t] = cplx(gs.next(), 0.0);
    fft3(c, f1, f2, f3, -1);
    fft3(x, f1, f2, f3, -1);
    // Xk <- Xk * sqrt(|Re Ck|) (CR:303-310); the filter is real and even, so the sign convention
    // of the transform does not matter
    for (size_t t = 0; t < nt; ++t) x[t] *= std::sqrt(std::fabs(c[t].real()));
    fft3(x, f1, f2, f3, +1);
    const double scale = 1.0 / (double)nt;
    for (int k = 0; k < n3; ++k)
        for (int j = 0; j < n2; ++j)
            for (int i = 0; i < n1; ++i) {
                double v = x[((size_t)k * f2 + j) * f1 + i].real() * scale;
                if (do_uniform)  // CR:333-341
                    v = (2.0 * (1.0 - 0.5 * erfcc(v / std::sqrt(2.0))) - 1.0) * max_value;
                out[((size_t)k * n2 + j) * n1 + i] = v;
            }
    return J1J2C_OK;
}

int j1j2c_setup_vacancies(int32_t seed, int32_t L, int32_t H, double pp, double pph, double ppv,
                          int32_t mode, int8_t* occu, int8_t* jh, int8_t* jv)
{
    if (L < 1 || H < 1 || !occu || !jh || !jv || (mode != 0 && mode != 1)) return J1J2C_EINVAL;
    const int L2 = L * L, N = L2 * H;
    Kiss k;
    k.seed(seed);
    int nimp = 0;
    if (mode == 0) {
        for (int i = 0; i < N; ++i) {
            const bool vac = k.next() < pp;
            occu[i] = vac ? 0 : 1;
            nimp += vac;
        }
    } else {
        // anticorrelated: remove random sites whose four in-plane neighbours are occupied
        for (int i = 0; i < N; ++i) occu[i] = 1;
        auto nb = [&](int i, int d) {
            const int z = i / L2, y = (i % L2) / L, x = i % L;
            int xx = x, yy = y;
            if (d == 0) yy = (y + 1) % L;
            if (d == 1) yy = (y + L - 1) % L;
            if (d == 2) xx = (x + 1) % L;
            if (d == 3) xx = (x + L - 1) % L;
            return xx + L * yy + L2 * z;
        };
        const int max_trials = 25 * N;
        for (int trials = 0; (double)nimp < pp * N && trials < max_trials; ++trials) {
            const int i = (int)(N * k.next());
            if (occu[i] * occu[nb(i, 0)] * occu[nb(i, 1)] * occu[nb(i, 2)] * occu[nb(i, 3)] == 1) {
                occu[i] = 0;
                ++nimp;
            }
        }
    }
    for (int i = 0; i < N; ++i) jh[i] = (k.next() < pph) ? 0 : 1;
    for (int i = 0; i < N; ++i) jv[i] = (k.next() < ppv) ? 0 : 1;
    return nimp;
}

int j1j2c_kiss_spins(int32_t seed, int32_t L, int32_t H, int32_t start, int32_t axis, int8_t* s)
{
    if (L < 1 || H < 1 || !s || start < 0 || start > 2) return J1J2C_EINVAL;
    const int L2 = L * L, N = L2 * H;
    if (start == J1J2C_START_HOT) {
        Kiss k;
        k.seed(seed);
        for (int i = 0; i < N; ++i) s[i] = (k.next() < 0.5) ? 1 : -1;
    } else if (start == J1J2C_START_FER) {
        for (int i = 0; i < N; ++i) s[i] = 1;
    } else {
        for (int i = 0; i < N; ++i) {
            const int x = i % L, y = (i % L2) / L;
            s[i] = (((axis == J1J2C_AXIS_X) ? y : x) & 1) ? -1 : 1;
        }
    }
    return J1J2C_OK;
}

int j1j2c_ladder(int32_t n, double tmin, double tmax, int32_t split, double tmid, double tfrac,
                 double* temps)
{
    if (n < 1 || !temps || tmax < tmin) return J1J2C_EINVAL;
    const int ninterval = n - 1;
    if (split && ninterval > 0) {
        if (n < 3 || !(tmid > tmin && tmid < tmax) || !(tfrac > 0.0 && tfrac < 1.0))
            return J1J2C_EINVAL;
        int nlow = (int)std::lround(ninterval * tfrac);
        if (nlow > ninterval - 1) nlow = ninterval - 1;
        if (nlow < 1) nlow = 1;
        const int nhigh = ninterval - nlow;
        temps[0] = tmin;
        for (int it = 1; it <= nlow; ++it)
            temps[it] = tmin + (tmid - tmin) * (double)it / (double)nlow;
        for (int it = 1; it <= nhigh; ++it)
            temps[nlow + it] = tmid + (tmax - tmid) * (double)it / (double)nhigh;
    } else if (n <= 1) {
        temps[0] = tmin;
    } else {
        for (int it = 1; it <= n; ++it)
            temps[it - 1] = tmin + (tmax - tmin) * (double)(it - 1) / (double)(n - 1);
    }
    return J1J2C_OK;
}

}  // extern "C"
