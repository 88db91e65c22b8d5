/*
 * ORACLE — test infrastructure only (see oracle.h).  Compiled with -ffp-contract=off so every
 * FP64 expression rounds exactly as written, in the order the Fortran source writes it.
 *
 * Citations "J:" are sim/J1J2_6tv.f90 and "CR:" sim/corr_rand_3d.f90 of ShadowQFT/J1J2-public.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------------------------ */
/* KISS05: rkiss05 J:3614-3632, kissinit J:3634-3695 (identical copies CR:90-160).            */
/* Fortran INTEGER(4) arithmetic wraps; ishft(.., -k) is a logical shift: uint32 restates it.  */
/* ------------------------------------------------------------------------------------------ */
double or_kiss_u(uint32_t st[4])
{
    st[0] = 69069u * st[0] + 1327217885u;
    st[1] ^= st[1] << 13;
    st[1] ^= st[1] >> 17;
    st[1] ^= st[1] << 5;
    st[2] = 18000u * (st[2] & 65535u) + (st[2] >> 16);
    st[3] = 30903u * (st[3] & 65535u) + (st[3] >> 16);
    uint32_t kiss = (st[0] + st[1] + (st[2] << 16) + st[3]) >> 1;
    return (double)kiss * 4.656612873077392578e-10;
}

static int32_t pm_step(int32_t idum)
{
    /* Park-Miller minimal standard step with Schrage's factorisation (J:3662-3665) */
    int32_t k = idum / 127773;
    int64_t v = (int64_t)16807 * (idum - k * 127773) - (int64_t)2836 * k;
    int32_t r = (int32_t)v;
    if (r < 0) r += 2147483647;
    return r;
}

void or_kiss_init(uint32_t st[4], int32_t seed)
{
    int32_t idum = (int32_t)((uint32_t)seed * 1099087573u); /* 32-bit LCG shuffle, J:3656 */
    if (idum < 0 && idum != INT32_MIN) idum = -idum;        /* abs(); abs(INT_MIN) wraps   */
    if (idum == 0) idum = 1;
    if (idum >= 2147483647) idum = 2147483646;
    for (int t = 0; t < 4; t++) {
        idum = pm_step(idum);
        st[t] = (uint32_t)(idum < 1 ? idum + 1 : idum);
    }
    (void)or_kiss_u(st); /* rdum = rkiss05(), J:3693 */
}

void or_kiss_draw(int32_t seed, int32_t n, double *out)
{
    uint32_t st[4];
    or_kiss_init(st, seed);
    for (int32_t i = 0; i < n; i++) out[i] = or_kiss_u(st);
}

/* gkiss05 CR:48-76 (Marsaglia polar method, cached second deviate), gkissinit CR:78-85 */
typedef struct {
    uint32_t k[4];
    double gset;
    int iset;
} or_gkiss;

static double gkiss(or_gkiss *g)
{
    if (g->iset != 1) {
        double v1, v2, s;
        for (;;) {
            v1 = 2.0 * or_kiss_u(g->k) - 1.0;
            v2 = 2.0 * or_kiss_u(g->k) - 1.0;
            s = v1 * v1 + v2 * v2;
            if (s < 1.0 && s > 0.0) break;
        }
        double fac = sqrt(-2.0 * log(s) / s);
        g->gset = v1 * fac;
        g->iset = 1;
        return v2 * fac;
    }
    g->iset = 0;
    return g->gset;
}

void or_gkiss_fill(int32_t seed, int32_t n, double *out)
{
    or_gkiss g;
    g.iset = 0;
    g.gset = 0.0;
    or_kiss_init(g.k, seed);
    for (int32_t i = 0; i < n; i++) out[i] = gkiss(&g);
}

/* erfcc CR:31-43 (Numerical Recipes Chebyshev fit) */
double or_erfcc(double x)
{
    double z = fabs(x);
    double t = 1.0 / (1.0 + 0.5 * z);
    double poly = t * (1.00002368 + t * (.37409196 + t * (.09678418 + t * (-.18628806 +
                  t * (.27886807 + t * (-1.13520398 + t * (1.48851587 + t * (-.82215223 +
                  t * .17087277))))))));
    double r = t * exp(((-z * z) - 1.26551223) + poly);
    if (x < 0.0) r = 2.0 - r;
    return r;
}

/* ------------------------------------------------------------------------------------------ */
/* Model set-up                                                                               */
/* ------------------------------------------------------------------------------------------ */

/* Setup_neighbor_table J:532-586; slot k of m holds m(k+1) */
void or_neighbors(int32_t L, int32_t H, int32_t *m)
{
    int32_t L2 = L * L, N = L2 * H;
    for (int32_t iz = 0; iz < H; iz++)
        for (int32_t iy = 0; iy < L; iy++)
            for (int32_t ix = 0; ix < L; ix++) {
                int32_t i = L * iy + ix + L2 * iz;
                m[0 * N + i] = (iy == L - 1) ? i - L * (L - 1) : i + L;
                m[1 * N + i] = (iy == 0) ? i + L * (L - 1) : i - L;
                m[2 * N + i] = (ix == L - 1) ? i - (L - 1) : i + 1;
                m[3 * N + i] = (ix == 0) ? i + (L - 1) : i - 1;
                m[8 * N + i] = (iz == H - 1) ? i - L2 * (H - 1) : i + L2;
                m[9 * N + i] = (iz == 0) ? i + L2 * (H - 1) : i - L2;
            }
    for (int32_t i = 0; i < N; i++) {
        m[4 * N + i] = m[2 * N + m[0 * N + i]];
        m[5 * N + i] = m[3 * N + m[0 * N + i]];
        m[6 * N + i] = m[2 * N + m[1 * N + i]];
        m[7 * N + i] = m[3 * N + m[1 * N + i]];
    }
}

/* Setup_vacancies J:1111-1165 after kissinit(seed) (J:317-319); mode 0 = RAN, 1 = COR */
int32_t or_setup_vacancies(int32_t seed, int32_t L, int32_t H, double pp, double pph, double ppv,
                           int32_t mode, const int32_t *m, int8_t *occu, int8_t *jh, int8_t *jv)
{
    uint32_t st[4];
    int32_t N = L * L * H, nimp = 0;
    or_kiss_init(st, seed);
    if (mode == 0) {
        for (int32_t i = 0; i < N; i++) {
            if (or_kiss_u(st) < pp) {
                occu[i] = 0;
                nimp++;
            } else {
                occu[i] = 1;
            }
        }
    } else {
        for (int32_t i = 0; i < N; i++) occu[i] = 1;
        int32_t max_trials = 25 * N, trials = 0;
        while ((double)nimp < pp * N && trials < max_trials) {
            int32_t i = (int32_t)(N * or_kiss_u(st));
            if (occu[i] * occu[m[0 * N + i]] * occu[m[1 * N + i]] * occu[m[2 * N + i]] *
                    occu[m[3 * N + i]] == 1) {
                occu[i] = 0;
                nimp++;
            }
            trials++;
        }
    }
    for (int32_t i = 0; i < N; i++) jh[i] = (or_kiss_u(st) < pph) ? 0 : 1;
    for (int32_t i = 0; i < N; i++) jv[i] = (or_kiss_u(st) < ppv) ? 0 : 1;
    return nimp;
}

static void init_spin_array(uint32_t st[4], int32_t L, int32_t H, int32_t start, int32_t axis,
                            int8_t *s)
{
    /* Initialize_spin_array J:1179-1209; start 0 = HOT, 1 = FER, 2 = STR; axis 0 = X, 1 = Y */
    int32_t L2 = L * L, N = L2 * H;
    if (start == 0) {
        for (int32_t i = 0; i < N; i++) s[i] = (or_kiss_u(st) < 0.5) ? 1 : -1;
    } else if (start == 1) {
        for (int32_t i = 0; i < N; i++) s[i] = 1;
    } else {
        for (int32_t iz = 0; iz < H; iz++)
            for (int32_t iy = 0; iy < L; iy++)
                for (int32_t ix = 0; ix < L; ix++) {
                    int32_t i = L * iy + ix + L2 * iz;
                    int32_t par = (axis == 0) ? iy : ix;
                    s[i] = (par & 1) ? -1 : 1;
                }
    }
}

void or_init_spins(int32_t seed, int32_t L, int32_t H, int32_t start, int32_t axis, int8_t *s)
{
    uint32_t st[4];
    or_kiss_init(st, seed);
    init_spin_array(st, L, H, start, axis, s);
}

/* Setup_temperature_ladder J:928-962 (PT branch): LINEAR, or SPLIT around tmid */
void or_ladder(int32_t n, double tmin, double tmax, int32_t split, double tmid, double tfrac,
               double *temps)
{
    int32_t ninterval = n - 1;
    if (split && ninterval > 0) {
        int32_t nlow = (int32_t)lround(ninterval * tfrac);
        if (nlow > ninterval - 1) nlow = ninterval - 1;
        if (nlow < 1) nlow = 1;
        int32_t nhigh = ninterval - nlow;
        temps[0] = tmin;
        for (int32_t it = 1; it <= nlow; it++)
            temps[it] = tmin + (tmid - tmin) * (double)it / (double)nlow;
        for (int32_t it = 1; it <= nhigh; it++)
            temps[nlow + it] = tmid + (tmax - tmid) * (double)it / (double)nhigh;
    } else if (n <= 1) {
        temps[0] = tmin;
    } else {
        for (int32_t it = 1; it <= n; it++)
            temps[it - 1] = tmin + (tmax - tmin) * (double)(it - 1) / (double)(n - 1);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Reference arithmetic                                                                       */
/* ------------------------------------------------------------------------------------------ */

/* Compute_local_field J:2498-2541, same order of operations (no contraction) */
double or_field_ref(const or_lat *g, const int8_t *s, int32_t i, double *n_out)
{
    const int32_t N = g->N;
    const int32_t *m = g->m;
    double f = 0.0, n = 0.0;
    int32_t j;
    j = m[0 * N + i];
    if (g->occu[j] == 1) {
        f = f + (double)s[j] * g->J1v * (double)g->jv[i];
        n = n - (double)s[j];
        f = f - g->p[j] * (double)s[j];
    }
    j = m[1 * N + i];
    if (g->occu[j] == 1) {
        f = f + (double)s[j] * g->J1v * (double)g->jv[j];
        n = n - (double)s[j];
        f = f - g->p[j] * (double)s[j];
    }
    j = m[2 * N + i];
    if (g->occu[j] == 1) {
        f = f + (double)s[j] * g->J1h * (double)g->jh[i];
        n = n + (double)s[j];
        f = f + g->p[j] * (double)s[j];
    }
    j = m[3 * N + i];
    if (g->occu[j] == 1) {
        f = f + (double)s[j] * g->J1h * (double)g->jh[j];
        n = n + (double)s[j];
        f = f + g->p[j] * (double)s[j];
    }
    for (int k = 4; k < 8; k++) {
        j = m[k * N + i];
        if (g->occu[j] == 1) f = f + (double)s[j] * g->J2;
    }
    for (int k = 8; k < 10; k++) {
        j = m[k * N + i];
        if (g->occu[j] == 1) f = f + (double)s[j] * g->J3;
    }
    f = f + (g->p[i] * n);
    if (n_out) *n_out = n;
    return f;
}

/* Measurement J:2807-2842: out = {curmag, curen, curstrx, curstry} */
void or_measurement_ref(const or_lat *g, const int8_t *s, double out[4])
{
    double imag = 0.0, ien = 0.0, sx = 0.0, sy = 0.0;
    const int32_t L = g->L, L2 = g->L * g->L;
    for (int32_t iz = 0; iz < g->H; iz++)
        for (int32_t i2 = 0; i2 < L2; i2++) {
            int32_t i = i2 + L2 * iz;
            if (g->occu[i] != 1) continue;
            imag = imag + (double)s[i];
            double f = or_field_ref(g, s, i, NULL);
            ien = ien - (double)s[i] * f;
            sx = sx + (double)(s[i] * (((i2 % L) & 1) ? -1 : 1));
            sy = sy + (double)(s[i] * (((i2 / L) & 1) ? -1 : 1));
        }
    double nocc = (double)(g->N - g->nimp);
    out[0] = (1.0 * imag) / nocc;
    out[1] = (0.5 * ien) / nocc;
    out[2] = (1.0 * sx) / nocc;
    out[3] = (1.0 * sy) / nocc;
}

/* Spatial_mean_local_nematic J:1028-1048 */
double or_nbar_ref(const or_lat *g, const int8_t *s)
{
    const int32_t N = g->N;
    const int32_t *m = g->m;
    double sum = 0.0;
    int32_t occ = g->N - g->nimp;
    if (occ < 1) occ = 1;
    for (int32_t i = 0; i < N; i++) {
        if (g->occu[i] == 0) continue;
        int32_t a = m[2 * N + i], b = m[0 * N + i], c = m[3 * N + i], d = m[1 * N + i];
        double v = (double)(s[i] * s[a] * g->occu[a]) - (double)(s[i] * s[b] * g->occu[b]) +
                   (double)(s[i] * s[c] * g->occu[c]) - (double)(s[i] * s[d] * g->occu[d]);
        sum = sum + v;
    }
    return sum / (double)occ;
}

/* Metro_sweep J:2544-2608 with Build_sweep_site_order J:2477-2495; obs = {mag, en, strx, stry} */
void or_metro_sweep_ref(const or_lat *g, int8_t *s, double beta, int32_t *flipcounts,
                        double obs[4], uint32_t kiss[4], int32_t rnd_order, int32_t *order)
{
    const int32_t N = g->N, L = g->L, L2 = g->L * g->L;
    if (order) {
        for (int32_t k = 0; k < N; k++) order[k] = k;
        if (rnd_order) {
            for (int32_t k = N - 1; k >= 1; k--) {
                int32_t j = (int32_t)((k + 1) * or_kiss_u(kiss));
                int32_t t = order[k];
                order[k] = order[j];
                order[j] = t;
            }
        }
    }
    double norm = (double)(N - g->nimp);
    for (int32_t k = 0; k < N; k++) {
        int32_t i = order ? order[k] : k;
        if (g->occu[i] != 1) continue;
        double field = or_field_ref(g, s, i, NULL);
        int8_t sold = s[i];
        double dmag = -2.0 * (double)sold / norm;
        double den = 2.0 * (double)sold * field / norm;
        int32_t i2 = i % L2;
        double dsx = dmag * ((((i2 % L) & 1) == 0) ? 1.0 : -1.0);
        double dsy = dmag * ((((i2 / L) & 1) == 0) ? 1.0 : -1.0);
        int flip;
        if (sold == 1)
            flip = (field <= 0.0) || (or_kiss_u(kiss) < exp(-(2.0 * field * beta)));
        else
            flip = (field >= 0.0) || (or_kiss_u(kiss) < exp(2.0 * field * beta));
        if (flip) {
            s[i] = (int8_t)(-s[i]);
            if (flipcounts) flipcounts[i]++;
            obs[0] += dmag;
            obs[1] += den;
            obs[2] += dsx;
            obs[3] += dsy;
        }
    }
}

static void slot_accumulate(double *S, double amag, double aen, double ax, double ay, double anb)
{
    /* per-slot running sums, Pt_measurement_loop J:1480-1513 */
    double x2 = ax * ax, y2 = ay * ay;
    double str2 = x2 + y2;
    double absstr = sqrt(str2);
    double nem = fabs(y2 - x2);
    double m2 = amag * amag, nb2 = anb * anb;
    S[0] += amag;
    S[1] += fabs(amag);
    S[2] += m2;
    S[3] += m2 * m2;
    S[4] += aen;
    S[5] += aen * aen;
    S[6] += fabs(ax);
    S[7] += fabs(ay);
    S[8] += x2;
    S[9] += x2 * x2;
    S[10] += y2;
    S[11] += y2 * y2;
    S[12] += str2;
    S[13] += str2 * str2;
    S[14] += absstr;
    S[15] += nem;
    S[16] += anb;
    S[17] += fabs(anb);
    S[18] += nb2;
    S[19] += nb2 * nb2;
    if (aen < S[20]) S[20] = aen;
    S[21] = aen;
}

/* PT SERIAL for one disorder configuration: Initialize_pt_state J:1218-1247,
 * Pt_equilibration_loop J:1250-1279, Pt_cycle J:1282-1300, Pt_attempt_swaps J:1303-1338,
 * Pt_measurement_loop accumulation J:1341-1524.  One KISS stream, consumed in reference order. */
typedef struct {
    const or_lat *g;
    int32_t nrep, ptswapever;
    const double *beta;
    int8_t *s;
    int32_t *rat, *tor;
    double *mag, *en, *sx, *sy, *nb;
    uint32_t kiss[4];
    int64_t *att, *acc;
} pt_state;

static void pt_cycle_ref(pt_state *P, int32_t phase)
{
    const int32_t N = P->g->N;
    for (int32_t slot = 0; slot < P->nrep; slot++) {
        int32_t rep = P->rat[slot];
        double obs[4] = {P->mag[rep], P->en[rep], P->sx[rep], P->sy[rep]};
        for (int32_t k = 0; k < P->ptswapever; k++)
            or_metro_sweep_ref(P->g, P->s + (size_t)rep * N, P->beta[slot], NULL, obs, P->kiss, 0,
                               NULL);
        P->mag[rep] = obs[0];
        P->en[rep] = obs[1];
        P->sx[rep] = obs[2];
        P->sy[rep] = obs[3];
    }
    int32_t start = (phase == 1) ? 0 : 1;
    double nocc = (double)(N - P->g->nimp);
    for (int32_t slot = start; slot < P->nrep - 1; slot += 2) {
        int32_t lo = P->rat[slot], hi = P->rat[slot + 1];
        P->att[slot]++;
        double tlo = P->en[lo] * nocc, thi = P->en[hi] * nocc;
        double delta = (P->beta[slot] - P->beta[slot + 1]) * (tlo - thi);
        if (delta >= 0.0 || or_kiss_u(P->kiss) < exp(delta)) {
            P->acc[slot]++;
            P->rat[slot] = hi;
            P->rat[slot + 1] = lo;
            P->tor[lo] = slot + 1;
            P->tor[hi] = slot;
        }
    }
}

void or_pt_serial_ref(const or_lat *g, int32_t nrep, const double *beta, int32_t ptswapever,
                      int32_t neq, int32_t nmess, int32_t irinit, int32_t iconf, int32_t start,
                      int32_t axis, double *sums, int64_t *attempts, int64_t *accepts,
                      int32_t *visitboth, int8_t *spins_out, int32_t *rep_at_temp_out)
{
    const int32_t N = g->N;
    pt_state P;
    P.g = g;
    P.nrep = nrep;
    P.ptswapever = ptswapever;
    P.beta = beta;
    P.s = spins_out;
    P.rat = (int32_t *)malloc(sizeof(int32_t) * nrep);
    P.tor = (int32_t *)malloc(sizeof(int32_t) * nrep);
    P.mag = (double *)malloc(sizeof(double) * nrep * 5);
    P.en = P.mag + nrep;
    P.sx = P.en + nrep;
    P.sy = P.sx + nrep;
    P.nb = P.sy + nrep;
    P.att = attempts;
    P.acc = accepts;
    for (int32_t k = 0; k < nrep - 1; k++) attempts[k] = accepts[k] = 0;
    for (int32_t rep = 0; rep < nrep; rep++) {
        P.rat[rep] = rep;
        P.tor[rep] = rep;
        or_kiss_init(P.kiss, irinit + (iconf - 1) * nrep + (rep + 1));
        init_spin_array(P.kiss, g->L, g->H, start, axis, P.s + (size_t)rep * N);
    }
    or_kiss_init(P.kiss, irinit + 100000 + iconf);

    double o[4];
    for (int32_t rep = 0; rep < nrep; rep++) {
        or_measurement_ref(g, P.s + (size_t)rep * N, o);
        P.mag[rep] = o[0];
        P.en[rep] = o[1];
        P.sx[rep] = o[2];
        P.sy[rep] = o[3];
    }
    int32_t phase = 1;
    for (int32_t c = 0; c < neq; c++) {
        pt_cycle_ref(&P, phase);
        phase = (phase == 1) ? 2 : 1;
    }
    /* measurement loop re-initialises the incremental observables (J:1432-1436) */
    for (int32_t rep = 0; rep < nrep; rep++) {
        or_measurement_ref(g, P.s + (size_t)rep * N, o);
        P.mag[rep] = o[0];
        P.en[rep] = o[1];
        P.sx[rep] = o[2];
        P.sy[rep] = o[3];
        P.nb[rep] = or_nbar_ref(g, P.s + (size_t)rep * N);
    }
    for (int32_t sl = 0; sl < nrep; sl++) {
        for (int32_t k = 0; k < OR_NSUM; k++) sums[sl * OR_NSUM + k] = 0.0;
        sums[sl * OR_NSUM + 20] = HUGE_VAL;
    }
    uint8_t *vc = (uint8_t *)calloc(nrep, 1), *vh = (uint8_t *)calloc(nrep, 1);
    phase = 1;
    for (int32_t c = 0; c < nmess; c++) {
        pt_cycle_ref(&P, phase);
        for (int32_t rep = 0; rep < nrep; rep++) {
            if (P.tor[rep] == 0) vc[rep] = 1;
            if (P.tor[rep] == nrep - 1) vh[rep] = 1;
            P.nb[rep] = or_nbar_ref(g, P.s + (size_t)rep * N);
        }
        for (int32_t sl = 0; sl < nrep; sl++) {
            int32_t rep = P.rat[sl];
            slot_accumulate(sums + sl * OR_NSUM, P.mag[rep], P.en[rep], P.sx[rep], P.sy[rep],
                            P.nb[rep]);
        }
        phase = (phase == 1) ? 2 : 1;
    }
    int32_t vb = 0;
    for (int32_t rep = 0; rep < nrep; rep++) vb += (vc[rep] && vh[rep]);
    *visitboth = vb;
    if (rep_at_temp_out)
        for (int32_t k = 0; k < nrep; k++) rep_at_temp_out[k] = P.rat[k];
    free(vc);
    free(vh);
    free(P.rat);
    free(P.tor);
    free(P.mag);
}

/* LOCAL sampler at one temperature: Equilibration_loop J:2122-2138 and Measurement_loop
 * J:2141-2216 (per-sweep lists; Process_data's averaging is done by the caller) */
void or_local_ref(const or_lat *g, const int8_t *s0, double beta, int32_t neq, int32_t nmess,
                  uint32_t kiss[4], double *maglist, double *enlist, double *strxlist,
                  double *strylist, double *nbarlist, int8_t *s_out)
{
    memcpy(s_out, s0, (size_t)g->N);
    double obs[4];
    or_measurement_ref(g, s_out, obs);
    for (int32_t k = 0; k < neq; k++) or_metro_sweep_ref(g, s_out, beta, NULL, obs, kiss, 0, NULL);
    or_measurement_ref(g, s_out, obs);
    for (int32_t k = 0; k < nmess; k++) {
        or_metro_sweep_ref(g, s_out, beta, NULL, obs, kiss, 0, NULL);
        maglist[k] = obs[0];
        enlist[k] = obs[1];
        strxlist[k] = obs[2];
        strylist[k] = obs[3];
        nbarlist[k] = or_nbar_ref(g, s_out);
    }
}

/* CPU throughput of the reference restatement: one independent PT ladder per thread
 * (mirrors the reference's rank-per-configuration layout, J:287-301).  Each thread initialises
 * its ladder, then times ncycles measurement-loop cycles (sweeps, swaps, nbar, slot sums:
 * J:1428-1524); the slowest thread's cycle time is returned in seconds. */
typedef struct {
    const or_lat *g;
    int32_t nrep, ptswapever, ncycles, seed;
    const double *beta;
    double seconds;
} bench_arg;

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* One ladder of the benchmark: spins from KISS HOT starts (seed + replica), observables, the
 * swap stream after seed + 100000, running sums by slot */
typedef struct {
    pt_state P;
    double *sums;
    int32_t phase;
} bench_ladder;

static void bench_ladder_init(bench_ladder *b, const or_lat *g, int32_t nrep, int32_t ptswapever,
                              const double *beta, int32_t seed)
{
    const int32_t N = g->N;
    pt_state *P = &b->P;
    P->g = g;
    P->nrep = nrep;
    P->ptswapever = ptswapever;
    P->beta = beta;
    P->s = (int8_t *)malloc((size_t)N * nrep);
    P->rat = (int32_t *)malloc(sizeof(int32_t) * nrep);
    P->tor = (int32_t *)malloc(sizeof(int32_t) * nrep);
    P->mag = (double *)malloc(sizeof(double) * nrep * 5);
    P->en = P->mag + nrep;
    P->sx = P->en + nrep;
    P->sy = P->sx + nrep;
    P->nb = P->sy + nrep;
    P->att = (int64_t *)calloc(nrep, sizeof(int64_t));
    P->acc = (int64_t *)calloc(nrep, sizeof(int64_t));
    b->sums = (double *)calloc((size_t)OR_NSUM * nrep, sizeof(double));
    for (int32_t rep = 0; rep < nrep; rep++) {
        P->rat[rep] = P->tor[rep] = rep;
        or_kiss_init(P->kiss, seed + rep);
        init_spin_array(P->kiss, g->L, g->H, 0, 0, P->s + (size_t)rep * N);
        double o[4];
        or_measurement_ref(g, P->s + (size_t)rep * N, o);
        P->mag[rep] = o[0];
        P->en[rep] = o[1];
        P->sx[rep] = o[2];
        P->sy[rep] = o[3];
    }
    or_kiss_init(P->kiss, seed + 100000);
    b->phase = 1;
}

/* ncycles measurement-loop cycles (sweeps, swaps, nbar, slot sums: J:1428-1524) */
static void bench_ladder_cycles(bench_ladder *b, int32_t ncycles)
{
    pt_state *P = &b->P;
    const int32_t N = P->g->N, nrep = P->nrep;
    for (int32_t c = 0; c < ncycles; c++) {
        pt_cycle_ref(P, b->phase);
        for (int32_t rep = 0; rep < nrep; rep++)
            P->nb[rep] = or_nbar_ref(P->g, P->s + (size_t)rep * N);
        for (int32_t sl = 0; sl < nrep; sl++) {
            int32_t rep = P->rat[sl];
            slot_accumulate(b->sums + sl * OR_NSUM, P->mag[rep], P->en[rep], P->sx[rep],
                            P->sy[rep], P->nb[rep]);
        }
        b->phase = (b->phase == 1) ? 2 : 1;
    }
}

static void bench_ladder_free(bench_ladder *b)
{
    free(b->sums);
    free(b->P.att);
    free(b->P.acc);
    free(b->P.s);
    free(b->P.rat);
    free(b->P.tor);
    free(b->P.mag);
}

static void *bench_worker(void *vp)
{
    bench_arg *a = (bench_arg *)vp;
    bench_ladder b;
    bench_ladder_init(&b, a->g, a->nrep, a->ptswapever, a->beta, a->seed);
    double t0 = now_s();
    bench_ladder_cycles(&b, a->ncycles);
    a->seconds = now_s() - t0;
    bench_ladder_free(&b);
    return NULL;
}

double or_bench_pt_ref(const or_lat *g, int32_t nthreads, int32_t nrep, const double *beta,
                       int32_t ptswapever, int32_t ncycles, int32_t irinit)
{
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    bench_arg *args = (bench_arg *)malloc(sizeof(bench_arg) * nthreads);
    for (int32_t t = 0; t < nthreads; t++) {
        args[t].g = g;
        args[t].nrep = nrep;
        args[t].ptswapever = ptswapever;
        args[t].ncycles = ncycles;
        args[t].seed = irinit + 1000 * t;
        args[t].beta = beta;
        args[t].seconds = 0.0;
        pthread_create(&th[t], NULL, bench_worker, &args[t]);
    }
    double worst = 0.0;
    for (int32_t t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        if (args[t].seconds > worst) worst = args[t].seconds;
    }
    free(th);
    free(args);
    return worst;
}

/* The same over nlad ladders, one disorder configuration each (gs[k]), on nthreads threads:
 * ladder k belongs to thread k % nthreads (the reference's configurations round-robin over
 * ranks, J:287-301).  Every thread first initialises its ladders; after a barrier the wall time
 * of ncycles cycles of every ladder is measured (until the last thread finishes) and returned in
 * seconds. */
typedef struct {
    const or_lat *const *gs;
    int32_t nlad, nthreads, t, nrep, ptswapever, ncycles, irinit;
    const double *beta;
    pthread_barrier_t *start;
    double done;
} bench_multi_arg;

static void *bench_multi_worker(void *vp)
{
    bench_multi_arg *a = (bench_multi_arg *)vp;
    int32_t mine = 0;
    for (int32_t k = a->t; k < a->nlad; k += a->nthreads) mine++;
    bench_ladder *b = (bench_ladder *)malloc(sizeof(bench_ladder) * (mine > 0 ? mine : 1));
    int32_t j = 0;
    for (int32_t k = a->t; k < a->nlad; k += a->nthreads, j++)
        bench_ladder_init(&b[j], a->gs[k], a->nrep, a->ptswapever, a->beta, a->irinit + 1000 * k);
    pthread_barrier_wait(a->start);
    for (j = 0; j < mine; j++) bench_ladder_cycles(&b[j], a->ncycles);
    a->done = now_s();
    for (j = 0; j < mine; j++) bench_ladder_free(&b[j]);
    free(b);
    return NULL;
}

double or_bench_pt_multi(const or_lat *const *gs, int32_t nlad, int32_t nthreads, int32_t nrep,
                         const double *beta, int32_t ptswapever, int32_t ncycles, int32_t irinit)
{
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    bench_multi_arg *args = (bench_multi_arg *)malloc(sizeof(bench_multi_arg) * nthreads);
    pthread_barrier_t start;
    pthread_barrier_init(&start, NULL, (unsigned)nthreads + 1u);
    for (int32_t t = 0; t < nthreads; t++) {
        args[t] = (bench_multi_arg){gs, nlad, nthreads, t, nrep, ptswapever, ncycles, irinit,
                                    beta, &start, 0.0};
        pthread_create(&th[t], NULL, bench_multi_worker, &args[t]);
    }
    pthread_barrier_wait(&start);
    const double t0 = now_s();
    double last = t0;
    for (int32_t t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        if (args[t].done > last) last = args[t].done;
    }
    pthread_barrier_destroy(&start);
    free(th);
    free(args);
    return last - t0;
}

/* ------------------------------------------------------------------------------------------ */
/* Replay of the device engine (colour order, Philox stream, own exp, fixed-point energy)      */
/* ------------------------------------------------------------------------------------------ */

/* Philox4x32-10, Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as easy as 1, 2, 3"
 * (SC'11): multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85. */
void or_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* The engine's own FP64 exponential, restated: Cody-Waite reduction x = k ln2 + r with ln2
 * split into a 32-bit head and a tail, degree-13 Taylor polynomial of e^r in Horner form with
 * fused multiply-adds, and an exact two-step scaling by 2^k.  Every step is an IEEE operation
 * with a single rounding, so the result is identical wherever it is evaluated. */
double or_dexp(double x)
{
    if (x != x) return x;
    if (x > 709.8) return HUGE_VAL;
    if (x < -745.2) return 0.0;
    const double inv_ln2 = 0x1.71547652b82fep+0;
    const double ln2_hi = 0x1.62e42fee00000p-1;
    const double ln2_lo = 0x1.a39ef35793c76p-33;
    double kd = nearbyint(x * inv_ln2);
    double r = fma(-kd, ln2_hi, x);
    r = fma(-kd, ln2_lo, r);
    double q = 0x1.6124613a86d09p-33; /* 1/13! */
    q = fma(q, r, 0x1.1eed8eff8d898p-29);
    q = fma(q, r, 0x1.ae64567f544e4p-26);
    q = fma(q, r, 0x1.27e4fb7789f5cp-22);
    q = fma(q, r, 0x1.71de3a556c734p-19);
    q = fma(q, r, 0x1.a01a01a01a01ap-16);
    q = fma(q, r, 0x1.a01a01a01a01ap-13);
    q = fma(q, r, 0x1.6c16c16c16c17p-10);
    q = fma(q, r, 0x1.1111111111111p-7);
    q = fma(q, r, 0x1.5555555555555p-5);
    q = fma(q, r, 0x1.5555555555555p-3);
    q = fma(q, r, 0.5);
    q = fma(q, r, 1.0);
    q = fma(q, r, 1.0);
    int32_t k = (int32_t)kd;
    int32_t k1 = k / 2, k2 = k - k1;
    uint64_t b1 = (uint64_t)(int64_t)(k1 + 1023) << 52, b2 = (uint64_t)(int64_t)(k2 + 1023) << 52;
    double s1, s2;
    memcpy(&s1, &b1, 8);
    memcpy(&s2, &b2, 8);
    return (q * s1) * s2;
}

static inline uint32_t philox_word(uint32_t seed, uint32_t conf, uint32_t c0, uint32_t c1,
                                   uint32_t c2, uint32_t tag, int w)
{
    uint32_t ctr[4] = {c0, c1, c2, tag}, key[2] = {seed, conf}, out[4];
    or_philox(ctr, key, out);
    return out[w];
}

/* Site -> Philox group: colour c = (x&1)|(y&1)<<1|(z&1)<<2, compact X=x>>1, Y=y>>1, Z=z>>1,
 * group g = ((c*Hh + Z)*Lh + Y)*Qr + (X>>2) with Qr = ceil(Lh/4), output word X&3. */
static inline void site_group(int32_t L, int32_t H, int32_t x, int32_t y, int32_t z, uint32_t *g,
                              int *w)
{
    int32_t Lh = L / 2, Hh = H / 2, Qr = (Lh + 3) / 4;
    int32_t c = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
    int32_t X = x >> 1, Y = y >> 1, Z = z >> 1;
    *g = (uint32_t)((((c * Hh + Z) * Lh + Y) * Qr) + (X >> 2));
    *w = X & 3;
}

#define TAG_SWEEP 0u
#define TAG_SWAP 1u
#define TAG_INIT 2u

/* flipcounts (may be NULL): per-site accepted flips, as Metro_sweep's flipcounts (J:2575) */
int64_t or_replay_sweeps(const or_lat *g, int8_t *s, double beta, uint32_t seed, uint32_t conf,
                         uint32_t rep, uint32_t sweep0, int32_t nsweeps, int32_t *flipcounts)
{
    const int32_t L = g->L, H = g->H, L2 = L * L;
    int64_t flips = 0;
    for (int32_t t = 0; t < nsweeps; t++) {
        uint32_t sweep = sweep0 + (uint32_t)t;
        for (int32_t c = 0; c < 8; c++) {
            int32_t cx = c & 1, cy = (c >> 1) & 1, cz = (c >> 2) & 1;
            for (int32_t z = cz; z < H; z += 2)
                for (int32_t y = cy; y < L; y += 2)
                    for (int32_t x = cx; x < L; x += 2) {
                        int32_t i = x + L * y + L2 * z;
                        if (g->occu[i] != 1) continue;
                        double field = or_field_ref(g, s, i, NULL);
                        int flip;
                        if (s[i] == 1 ? field <= 0.0 : field >= 0.0) {
                            flip = 1;
                        } else {
                            uint32_t gi;
                            int w;
                            site_group(L, H, x, y, z, &gi, &w);
                            uint32_t r = philox_word(seed, conf, rep, sweep, gi, TAG_SWEEP, w);
                            /* FP64 uniform: the word rotated left by 9, times 2^-32 */
                            double u = (double)((r << 9) | (r >> 23)) * 0x1p-32;
                            double t2 = (2.0 * field) * beta;
                            flip = u < or_dexp(s[i] == 1 ? -t2 : t2);
                        }
                        if (flip) {
                            s[i] = (int8_t)(-s[i]);
                            flips++;
                            if (flipcounts) flipcounts[i]++;
                        }
                    }
        }
    }
    return flips;
}

/* Fixed-point energy: each occupied site adds llrint(-s_i*field_i * 2^32) to an int64, so the
 * lattice total is independent of summation order; E_total = acc * 2^-33 (the 1/2 of J:2840).
 * ints = {sum s, sum s(-1)^x, sum s(-1)^y, sum s*(s_+x + s_-x - s_+y - s_-y)};
 * obs  = {mag, en (per occupied site), strx, stry, nbar} exactly as J:2833-2841, J:1047. */
void or_replay_measure(const or_lat *g, const int8_t *s, int64_t ints[4], int64_t *eacc,
                       double obs[5])
{
    const int32_t N = g->N, L = g->L, L2 = L * L;
    const int32_t *m = g->m;
    int64_t M = 0, SX = 0, SY = 0, NB = 0, acc = 0;
    for (int32_t i = 0; i < N; i++) {
        if (g->occu[i] != 1) continue;
        int32_t si = s[i];
        double f = or_field_ref(g, s, i, NULL);
        double e = -((double)si * f);
        acc += llrint(e * 4294967296.0);
        int32_t i2 = i % L2;
        M += si;
        SX += ((i2 % L) & 1) ? -si : si;
        SY += ((i2 / L) & 1) ? -si : si;
        int32_t a = m[2 * N + i], b = m[0 * N + i], c = m[3 * N + i], d = m[1 * N + i];
        NB += si * (s[a] * g->occu[a] - s[b] * g->occu[b] + s[c] * g->occu[c] -
                    s[d] * g->occu[d]);
    }
    ints[0] = M;
    ints[1] = SX;
    ints[2] = SY;
    ints[3] = NB;
    *eacc = acc;
    if (obs) {
        int32_t nocc = N - g->nimp;
        double dn = (double)nocc;
        obs[0] = (double)M / dn;
        obs[1] = ((double)acc * 0x1p-33) / dn;
        obs[2] = (double)SX / dn;
        obs[3] = (double)SY / dn;
        obs[4] = (double)NB / (double)(nocc < 1 ? 1 : nocc);
    }
}

void or_replay_pt(const or_lat *g, int32_t nrep, const double *beta, int32_t ptswapever,
                  int32_t ncycles, uint32_t cycle0, uint32_t seed, uint32_t conf, int32_t measure,
                  int32_t phase0, int8_t *spins, int32_t *rep_at_temp, int32_t *temp_of_rep,
                  double *sums, int64_t *nmeas, int64_t *attempts, int64_t *accepts,
                  uint8_t *visited, double *obs_out, int32_t *flips)
{
    const int32_t N = g->N;
    double *obs = (double *)malloc(sizeof(double) * 5 * nrep);
    double *etot = (double *)malloc(sizeof(double) * nrep);
    int32_t phase = phase0;
    for (int32_t cyc = 0; cyc < ncycles; cyc++) {
        uint32_t cycle = cycle0 + (uint32_t)cyc;
        for (int32_t rep = 0; rep < nrep; rep++) {
            double b = beta[temp_of_rep[rep]];
            or_replay_sweeps(g, spins + (size_t)rep * N, b, seed, conf, (uint32_t)rep,
                             cycle * (uint32_t)ptswapever, ptswapever,
                             flips ? flips + (size_t)temp_of_rep[rep] * N : NULL);
            int64_t ints[4], acc;
            or_replay_measure(g, spins + (size_t)rep * N, ints, &acc, obs + 5 * rep);
            etot[rep] = (double)acc * 0x1p-33;
        }
        for (int32_t sl = (phase == 1) ? 0 : 1; sl < nrep - 1; sl += 2) {
            int32_t lo = rep_at_temp[sl], hi = rep_at_temp[sl + 1];
            attempts[sl]++;
            double delta = (beta[sl] - beta[sl + 1]) * (etot[lo] - etot[hi]);
            int acc = delta >= 0.0;
            if (!acc) {
                double u = (double)philox_word(seed, conf, cycle, (uint32_t)sl, 0u, TAG_SWAP, 0) *
                           0x1p-32;
                acc = u < or_dexp(delta);
            }
            if (acc) {
                accepts[sl]++;
                rep_at_temp[sl] = hi;
                rep_at_temp[sl + 1] = lo;
                temp_of_rep[lo] = sl + 1;
                temp_of_rep[hi] = sl;
            }
        }
        if (measure) {
            for (int32_t rep = 0; rep < nrep; rep++) {
                if (temp_of_rep[rep] == 0) visited[rep] |= 1;
                if (temp_of_rep[rep] == nrep - 1) visited[rep] |= 2;
            }
            for (int32_t sl = 0; sl < nrep; sl++) {
                const double *o = obs + 5 * rep_at_temp[sl];
                slot_accumulate(sums + sl * OR_NSUM, o[0], o[1], o[2], o[3], o[4]);
                nmeas[sl]++;
            }
        }
        phase = (phase == 1) ? 2 : 1;
    }
    if (obs_out) memcpy(obs_out, obs, sizeof(double) * 5 * nrep);
    free(obs);
    free(etot);
}

/* Wolff update of the engine, restated (FP64 form): bonds owned by each site (+x, +y,
 * (+x,+y), (-x,+y), +z = slots m3, m1, m5, m6, m9) with coupling K of Compute_local_field
 * (J:2498-2541); a bond with K s_i s_j > 0 is active when u < 1 - exp(-2 beta K s_i s_j), u from
 * word b of ctr = (rep, cycle, compact site index, 5) for the in-plane bonds b = 0..3 and from
 * word X & 3 of ctr = (rep, cycle, group, 67) for the +z bond; the component of the seed site
 * floor(w*N/2^32), w from ctr = (rep, cycle, 0xFFFFFFFF, 4), is flipped (no flip when the seed
 * is a vacancy).  Returns the flipped cluster size. */
static int32_t uf_find(int32_t *lab, int32_t x)
{
    while (lab[x] != x) {
        lab[x] = lab[lab[x]];
        x = lab[x];
    }
    return x;
}

int64_t or_wolff_step(const or_lat *g, int8_t *s, double beta, uint32_t seed, uint32_t conf,
                      uint32_t rep, uint32_t cycle)
{
    const int32_t N = g->N, L = g->L, H = g->H;
    const int32_t *m = g->m;
    static const int slot[5] = {2, 0, 4, 5, 8};
    int32_t *lab = (int32_t *)malloc(sizeof(int32_t) * N);
    for (int32_t i = 0; i < N; i++) lab[i] = i;
    for (int32_t i = 0; i < N; i++) {
        if (g->occu[i] != 1) continue;
        int32_t x = i % L, y = (i / L) % L, z = i / (L * L);
        uint32_t gi;
        int w;
        site_group(L, H, x, y, z, &gi, &w);
        const int32_t Lh = L / 2, Hh = H / 2;
        const int32_t cc = (x & 1) | ((y & 1) << 1) | ((z & 1) << 2);
        const uint32_t ci = (uint32_t)(((cc * Hh + (z >> 1)) * Lh + (y >> 1)) * Lh + (x >> 1));
        for (int b = 0; b < 5; b++) {
            int32_t j = m[slot[b] * N + i];
            if (g->occu[j] != 1) continue;
            double K;
            if (b == 0)
                K = ((g->jh[i] ? g->J1h : 0.0) + g->p[i]) + g->p[j];
            else if (b == 1)
                K = ((g->jv[i] ? g->J1v : 0.0) - g->p[i]) - g->p[j];
            else if (b < 4)
                K = g->J2;
            else
                K = g->J3;
            double wgt = (s[i] * s[j] > 0) ? K : -K;
            if (!(wgt > 0.0)) continue;
            uint32_t r = b < 4 ? philox_word(seed, conf, rep, cycle, ci, 5u, b)
                               : philox_word(seed, conf, rep, cycle, gi, 3u + 16u * 4u, w);
            double u = (double)((r << 9) | (r >> 23)) * 0x1p-32;
            double pa = 1.0 - or_dexp(-((2.0 * wgt) * beta));
            if (u < pa) {
                int32_t a = uf_find(lab, i), c = uf_find(lab, j);
                if (a != c) {
                    if (a < c) lab[c] = a;
                    else lab[a] = c;
                }
            }
        }
    }
    uint32_t wseed = philox_word(seed, conf, rep, cycle, 0xFFFFFFFFu, 4u, 0);
    int32_t site = (int32_t)(((uint64_t)wseed * (uint64_t)N) >> 32);
    int64_t count = 0;
    if (g->occu[site] == 1) {
        int32_t root = uf_find(lab, site);
        for (int32_t i = 0; i < N; i++)
            if (uf_find(lab, i) == root) {
                s[i] = (int8_t)(-s[i]);
                count++;
            }
    }
    free(lab);
    return count;
}

/* HOT start from the Philox stream: s = +1 when the site's word is below 2^31 (u < 1/2) */
void or_hot_spins_philox(int32_t L, int32_t H, uint32_t seed, uint32_t conf, uint32_t rep,
                         int8_t *s)
{
    for (int32_t z = 0; z < H; z++)
        for (int32_t y = 0; y < L; y++)
            for (int32_t x = 0; x < L; x++) {
                uint32_t gi;
                int w;
                site_group(L, H, x, y, z, &gi, &w);
                uint32_t r = philox_word(seed, conf, rep, 0u, gi, TAG_INIT, w);
                s[x + L * y + L * L * z] = (r < 0x80000000u) ? 1 : -1;
            }
}
