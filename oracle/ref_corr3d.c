/*
 * ORACLE — test infrastructure only.
 *
 * make_corr_rand_3d (sim/corr_rand_3d.f90:191-386) restated in C around the reference's own
 * vendored Ooura FFT (vendor/fft2d/fftsg3d.c + fftsg.c, compiled from the reference tree by
 * oracle/Makefile into oracle/_ref/).  This is the closest runnable form of the reference's
 * disorder generator here (the Fortran build needs a Fortran compiler); it produces the golden
 * disorder vectors in tests/golden/ that pin the numpy restatement and the engine's generator.
 *
 * Index mapping: the Fortran array x(0:n1-1,0:n2-1,0:n3-1) (i fastest) is the C array
 * a[k][j][i]; the Fortran rdft3d(n1max,n2max,n1,n2,n3,...) is the C rdft3d(n3,n2,n1,...) with
 * the innermost dimension padded by 2 for the sorted half spectrum (CR:229-230).
 */
#include <math.h>
#include <stdlib.h>

#include "oracle.h"

void rdft3d(int, int, int, int, double ***, double *, int *, double *);
void rdft3dsort(int, int, int, int, double ***);

static int nextpow2(int n)
{
    int p = 1;
    while (p < n) p *= 2; /* CR:350-357 */
    return p;
}

static double ***alloc3(int n1, int n2, int n3)
{
    double ***a = (double ***)malloc(sizeof(double **) * n1);
    double **rows = (double **)malloc(sizeof(double *) * n1 * n2);
    double *data = (double *)calloc((size_t)n1 * n2 * n3, sizeof(double));
    for (int i = 0; i < n1; i++) {
        a[i] = rows + (size_t)i * n2;
        for (int j = 0; j < n2; j++) a[i][j] = data + ((size_t)i * n2 + j) * n3;
    }
    return a;
}

static void free3(double ***a)
{
    free(a[0][0]);
    free(a[0]);
    free(a);
}

/* x[(k*n2 + j)*n1 + i] = x(i,j,k) of the Fortran routine */
void ref_make_corr_rand_3d(double *x, int n1, int n2, int n3, double xi, int seed, int do_uniform,
                           double max_value)
{
    int f1 = nextpow2(n1), f2 = nextpow2(n2), f3 = nextpow2(n3);
    int nw = f1 > f2 ? f1 : f2;
    nw = nw > f3 ? nw : f3;
    int *ip = (int *)calloc(2 + (int)sqrt((double)nw) + 16, sizeof(int));
    double *w = (double *)calloc(nw + 1024, sizeof(double));
    double ***c = alloc3(f3, f2, f1 + 2);
    double ***xw = alloc3(f3, f2, f1 + 2);

    /* correlation C(dx,dy,dz) = exp(-r/xi) with periodic distances, CR:261-268, CR:362-384 */
    for (int k = 0; k < f3; k++)
        for (int j = 0; j < f2; j++)
            for (int i = 0; i < f1; i++) {
                int dx = i < f1 - i ? i : f1 - i;
                int dy = j < f2 - j ? j : f2 - j;
                int dz = k < f3 - k ? k : f3 - k;
                double r = sqrt((double)(dx * dx + dy * dy + dz * dz));
                double corr;
                if (xi <= 0.0)
                    corr = (r == 0.0) ? 1.0 : 0.0;
                else
                    corr = exp(-r / xi);
                c[k][j][i] = corr;
            }
    ip[0] = 0;
    rdft3d(f3, f2, f1, 1, c, NULL, ip, w);
    rdft3dsort(f3, f2, f1, 1, c);

    /* white noise in Fortran order after gkissinit(seed), CR:256, CR:280-287 */
    double *noise = (double *)malloc(sizeof(double) * (size_t)f1 * f2 * f3);
    or_gkiss_fill(seed, f1 * f2 * f3, noise);
    size_t t = 0;
    for (int k = 0; k < f3; k++)
        for (int j = 0; j < f2; j++)
            for (int i = 0; i < f1; i++) xw[k][j][i] = noise[t++];
    free(noise);
    rdft3d(f3, f2, f1, 1, xw, NULL, ip, w);
    rdft3dsort(f3, f2, f1, 1, xw);

    /* Xk <- Xk * sqrt(|Ck|) on Re and Im, CR:303-310 */
    for (int k3 = 0; k3 < f3; k3++)
        for (int k2 = 0; k2 < f2; k2++)
            for (int k1 = 0; k1 <= f1 / 2; k1++) {
                double fac = sqrt(fabs(c[k3][k2][2 * k1]));
                xw[k3][k2][2 * k1] = xw[k3][k2][2 * k1] * fac;
                xw[k3][k2][2 * k1 + 1] = xw[k3][k2][2 * k1 + 1] * fac;
            }
    rdft3dsort(f3, f2, f1, -1, xw);
    rdft3d(f3, f2, f1, -1, xw, NULL, ip, w);

    double scale = 2.0 / (double)f1 / (double)f2 / (double)f3; /* CR:319 */
    for (int k = 0; k < n3; k++)
        for (int j = 0; j < n2; j++)
            for (int i = 0; i < n1; i++) {
                double v = xw[k][j][i] * scale;
                if (do_uniform) /* CR:333-341 */
                    v = (2.0 * (1.0 - 0.5 * or_erfcc(v / sqrt(2.0))) - 1.0) * max_value;
                x[((size_t)k * n2 + j) * n1 + i] = v;
            }
    free3(c);
    free3(xw);
    free(ip);
    free(w);
}
