/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C, FP64 restatement of PyTransit's RoadRunner evaluation path
 * (reference: hpparvi/PyTransit 2.8.1).  The tests check the CUDA library in
 * pytransit_gb300/ against it, and it is the CPU baseline timed beside it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may load
 * it; the product path never does.
 *
 * Compile with -ffp-contract=off: the reference runs numba/numpy without
 * fused multiply-adds, and BJD-scale phase folding is sensitive to the
 * rounding sequence at the 1e-10 d level.
 *
 * Pinned against tests/golden/*.npz, which were produced by running the
 * reference's own unmodified RoadRunner Python code (see
 * tests/golden/make_golden.py).  The orbit layer (meepmeep's solve2d /
 * sep_c / bounding_box) is absent from the reference; it is restated here
 * and in the golden shim from the same published algorithm, so RoadRunner
 * flux parity against real meepmeep is unpinned.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RRO_PI 3.141592653589793238462643383279502884

/* ------------------------------------------------------------------ */
/* Grids                                                               */
/* ------------------------------------------------------------------ */

/* numpy.linspace(start, stop, num) with endpoint=True:
 * y[i] = i*step + start, step = (stop-start)/(num-1), y[-1] = stop. */
void rro_linspace(double start, double stop, int num, double *out)
{
    if (num <= 0) return;
    if (num == 1) { out[0] = start; return; }
    double step = (stop - start) / (double)(num - 1);
    for (int i = 0; i < num; ++i) out[i] = (double)i * step + start;
    out[num - 1] = stop;
}

/* create_z_grid, pytransit/models/roadrunner/common.py:132-149.
 * z_means[0] stays 0 (never assigned in the reference). */
void rro_z_grid(double zcut, int nin, int nedge, double *ze, double *zm)
{
    int nz = nin + nedge;
    double mucut = sqrt(1.0 - zcut * zcut);
    double dz = zcut / nin;
    double dmu = mucut / nedge;
    for (int i = 0; i < nz; ++i) { ze[i] = 0.0; zm[i] = 0.0; }
    for (int i = 0; i < nin - 1; ++i) ze[i] = (i + 1) * dz;
    for (int i = 0; i < nedge + 1; ++i) {
        double m = i * dmu;
        ze[nz - i - 1] = sqrt(1.0 - m * m);
    }
    for (int i = 0; i < nz - 1; ++i) zm[i + 1] = 0.5 * (ze[i] + ze[i + 1]);
}

/* ------------------------------------------------------------------ */
/* Circle-circle intersection                                          */
/* ------------------------------------------------------------------ */

/* circle_circle_intersection_area, common.py:37-49 (two-arccos form). */
double rro_cci_acos(double r1, double r2, double b)
{
    if (r1 < b - r2) return 0.0;
    else if (r1 >= b + r2) return RRO_PI * r2 * r2;
    else if (b - r2 <= -r1) return RRO_PI * r1 * r1;
    return r2 * r2 * acos((b * b + r2 * r2 - r1 * r1) / (2 * b * r2)) +
           r1 * r1 * acos((b * b + r1 * r1 - r2 * r2) / (2 * b * r1)) -
           0.5 * sqrt((-b + r2 + r1) * (b + r2 - r1) * (b - r2 + r1) * (b + r2 + r1));
}

/* tsort, common.py:6-33: descending sort of three lengths. */
static void rro_tsort(double r1, double r2, double b, double *x, double *y, double *z)
{
    if (r1 > r2) {
        if (r1 > b) { *x = r1; if (r2 > b) { *y = r2; *z = b; } else { *y = b; *z = r2; } }
        else { *x = b; *y = r1; *z = r2; }
    } else {
        if (r2 > b) { *x = r2; if (r1 > b) { *y = r1; *z = b; } else { *y = b; *z = r1; } }
        else { *x = b; *y = r2; *z = r1; }
    }
}

/* circle_circle_intersection_area_kite, common.py:53-73 (Agol et al. 2020).
 * Returns the area; *kappa0 receives the second return value. */
double rro_ccia(double r1, double r2, double b, double *kappa0)
{
    double k0v;
    double area;
    if (r1 + r2 <= b) { area = 0.0; k0v = 0.0; }
    else if (fabs(r1 - r2) < b && b <= r1 + r2) {
        double x, y, z;
        rro_tsort(r1, r2, b, &x, &y, &z);
        double a_kite = 0.5 * sqrt((x + (y + z)) * (z - (x - y)) * (z + (x - y)) * (x + (y - z)));
        double k0 = atan2(2.0 * a_kite, (r2 - r1) * (r2 + r1) + b * b);
        double k1 = atan2(2.0 * a_kite, (r1 - r2) * (r1 + r2) + b * b);
        area = r1 * r1 * k1 + r2 * r2 * k0 - a_kite;
        k0v = k0;
    }
    else if (b <= r1 - r2) { area = RRO_PI * r2 * r2; k0v = RRO_PI; }
    else if (b <= r2 - r1) { area = RRO_PI * r1 * r1; k0v = 0.0; }
    else { area = NAN; k0v = NAN; }
    if (kappa0) *kappa0 = k0v;
    return area;
}

/* ------------------------------------------------------------------ */
/* Weight tables                                                       */
/* ------------------------------------------------------------------ */

/* One (k, g) row of calculate_weights_2d / _3d, common.py:173-184, 210-222. */
static void rro_weight_row(double k, double g, const double *ze, int nz, double *row)
{
    double b = g * (1.0 + k);
    double a0 = rro_cci_acos(ze[0], k, b);
    row[0] = a0;
    double s = row[0];
    for (int i = 1; i < nz; ++i) {
        double a1 = rro_cci_acos(ze[i], k, b);
        row[i] = a1 - a0;
        a0 = a1;
        s += row[i];
    }
    for (int i = 0; i < nz; ++i) row[i] /= s;
}

/* calculate_weights_2d, common.py:153-185.  W is [ng, nz]; returns dg. */
double rro_weights_2d(double k, const double *ze, int nz, int ng, double *W)
{
    double *gs = (double *)malloc(sizeof(double) * ng);
    rro_linspace(0.0, 1.0 - 1e-7, ng, gs);
    for (int ig = 0; ig < ng; ++ig) rro_weight_row(k, gs[ig], ze, nz, W + (size_t)ig * nz);
    double dg = gs[1] - gs[0];
    free(gs);
    return dg;
}

/* calculate_weights_3d, common.py:189-223.  W is [nk, ng, nz].
 * Writes dk = (k1-k0)/nk (grid spacing is (k1-k0)/(nk-1): reproduced as is)
 * and dg = gs[1]-gs[0]. */
void rro_weights_3d(int nk, double k0, double k1, const double *ze, int nz, int ng,
                    double *W, double *dk, double *dg)
{
    double *ks = (double *)malloc(sizeof(double) * nk);
    double *gs = (double *)malloc(sizeof(double) * ng);
    rro_linspace(k0, k1, nk, ks);
    rro_linspace(0.0, 1.0 - 1e-7, ng, gs);
    #pragma omp parallel for schedule(static)
    for (int ik = 0; ik < nk; ++ik)
        for (int ig = 0; ig < ng; ++ig)
            rro_weight_row(ks[ik], gs[ig], ze, nz, W + ((size_t)ik * ng + ig) * nz);
    *dk = (k1 - k0) / nk;
    *dg = gs[1] - gs[0];
    free(ks);
    free(gs);
}

/* interpolate_mean_limb_darkening_s, common.py:225-233.  The reference reads
 * lda[ng] for g in [1-1e-7, 1]; here the index is clamped to ng-2 (linear
 * extrapolation from the last cell), which is what the GPU path does too. */
double rro_interp_ldm(double g, double dg, const double *lda, int ng)
{
    if (g < 0.0) return NAN;
    if (g > 1.0) return 0.0;
    int i = (int)floor(g / dg);
    if (i > ng - 2) i = ng - 2;
    double a = (g - i * dg) / dg;
    return (1.0 - a) * lda[i] + a * lda[i + 1];
}

/* ------------------------------------------------------------------ */
/* Limb darkening laws, pytransit/models/numba/ldmodels.py:23-140     */
/* ------------------------------------------------------------------ */

enum {
    RRO_LD_UNIFORM = 0, RRO_LD_LINEAR = 1, RRO_LD_QUADRATIC = 2, RRO_LD_QUADRATIC_TRI = 3,
    RRO_LD_NONLINEAR = 4, RRO_LD_GENERAL = 5, RRO_LD_SQUARE_ROOT = 6, RRO_LD_LOGARITHMIC = 7,
    RRO_LD_EXPONENTIAL = 8, RRO_LD_POWER_2 = 9, RRO_LD_POWER_2_PM = 10
};

double rro_ld_value(int law, double mu, const double *pv, int npar)
{
    switch (law) {
    case RRO_LD_UNIFORM: return 1.0;
    case RRO_LD_LINEAR: return 1. - pv[0] * (1. - mu);
    case RRO_LD_QUADRATIC: return 1. - pv[0] * (1. - mu) - pv[1] * (1. - mu) * (1. - mu);
    case RRO_LD_QUADRATIC_TRI: {
        double a = sqrt(pv[0]), b = 2 * pv[1];
        double u = a * b, v = a * (1. - b);
        return 1. - u * (1. - mu) - v * (1. - mu) * (1. - mu);
    }
    case RRO_LD_NONLINEAR:
        return 1. - pv[0] * (1. - sqrt(mu)) - pv[1] * (1. - mu) - pv[2] * (1. - pow(mu, 1.5)) -
               pv[3] * (1. - mu * mu);
    case RRO_LD_GENERAL: {
        double s = 0.0;
        for (int i = 0; i < npar; ++i) s += pv[i] * (1.0 - pow(mu, (double)(i + 1)));
        return s;
    }
    case RRO_LD_SQUARE_ROOT: return 1. - pv[0] * (1. - mu) - pv[1] * (1. - sqrt(mu));
    case RRO_LD_LOGARITHMIC: return 1. - pv[0] * (1. - mu) - pv[1] * mu * log(mu);
    case RRO_LD_EXPONENTIAL: return 1. - pv[0] * (1. - mu) - pv[1] / (1. - exp(mu));
    case RRO_LD_POWER_2: return 1. - pv[0] * (1. - pow(mu, pv[1]));
    case RRO_LD_POWER_2_PM: {
        double c = 1 - pv[0] + pv[1];
        double a = log2(c / pv[1]);
        return 1. - c * (1. - pow(mu, a));
    }
    }
    return NAN;
}

/* Analytic disk integrals (ldi_*).  Returns 1 and writes *istar when the law
 * has one in the reference's RoadRunner law table, rrmodel.py:48-58. */
int rro_ld_integral(int law, const double *pv, double *istar)
{
    switch (law) {
    case RRO_LD_UNIFORM: *istar = RRO_PI; return 1;
    /* 2*pi*1/6*(3-2u): the reference's RoadRunner copy has 2u, not u. */
    case RRO_LD_LINEAR: *istar = 2 * RRO_PI * 1 / 6 * (3 - 2 * pv[0]); return 1;
    case RRO_LD_QUADRATIC: *istar = 2 * RRO_PI * 1 / 12 * (-2 * pv[0] - pv[1] + 6); return 1;
    case RRO_LD_QUADRATIC_TRI: {
        double a = sqrt(pv[0]), b = 2 * pv[1];
        double u = a * b, v = a * (1. - b);
        *istar = 2 * RRO_PI * 1 / 12 * (-2 * u - v + 6);
        return 1;
    }
    case RRO_LD_POWER_2:
        *istar = 2 * RRO_PI * (-pv[0] * pv[1] + pv[1] + 2) / (2 * pv[1] + 4);
        return 1;
    }
    return 0;
}

/* Numerical disk integral, rrmodel.py:222-227: 2*pi*trapezoid(z*I(mu(z)), z)
 * with mu = linspace(1, 0, 200), z = sqrt(1-mu^2). */
double rro_ld_integral_numeric(int law, const double *pv, int npar)
{
    enum { N = 200 };
    double mu[N], z[N], y[N];
    rro_linspace(1.0, 0.0, N, mu);
    for (int i = 0; i < N; ++i) {
        z[i] = sqrt(1 - mu[i] * mu[i]);
        y[i] = z[i] * rro_ld_value(law, mu[i], pv, npar);
    }
    double s = 0.0;
    for (int i = 0; i < N - 1; ++i) s += (z[i + 1] - z[i]) * (y[i + 1] + y[i]) / 2.0;
    return 2 * RRO_PI * s;
}

/* evaluate_ld / evaluate_ldi for a named law over a (npv, npb, npar) ldc array. */
void rro_evaluate_ld(int law, const double *mu, int nmu, const double *ldc, int npv, int npb,
                     int npar, double *ldp, double *istar)
{
    for (int ipv = 0; ipv < npv; ++ipv)
        for (int ipb = 0; ipb < npb; ++ipb) {
            const double *pv = ldc + ((size_t)ipv * npb + ipb) * npar;
            for (int j = 0; j < nmu; ++j)
                ldp[((size_t)ipv * npb + ipb) * nmu + j] = rro_ld_value(law, mu[j], pv, npar);
            double is;
            if (!rro_ld_integral(law, pv, &is)) is = rro_ld_integral_numeric(law, pv, npar);
            istar[(size_t)ipv * npb + ipb] = is;
        }
}

/* ------------------------------------------------------------------ */
/* Orbit layer: restatement of meepmeep.backends.numba.point2d         */
/* ------------------------------------------------------------------ */

/* Solve Kepler's equation E - e sin E = M by Newton's method as in
 * pytransit/orbits/orbits_py.py:145-154 (tolerance 1e-8, <=1000 steps). */
static double rro_ea_newton(double M, double e)
{
    double E = M, err = 0.05;
    int k = 0;
    while (fabs(err) > 1e-8 && k < 1000) {
        err = E - e * sin(E) - M;
        E = E - err / (1.0 - e * cos(E));
        k++;
    }
    return E;
}

/* solve2d(phase, p, a, i, e, w): Taylor coefficients (degree 4) of the
 * sky-projected planet position about t = phase, with t = 0 at conjunction
 * (true anomaly f = pi/2 - w, pytransit/orbits/orbits_py.py:83-86).
 * Layout c[0..4] = x, c[5..9] = y, x(t) = sum c[j] t^j
 * (pytransit/models/numba/gdmodel.py:441-442).  Sky axes as
 * pytransit/orbits/taylor_z.py:62-76: x = -r cos(w+f), y = -r sin(w+f) cos i.
 *
 * The derivatives are exact: the in-plane Keplerian state (position,
 * velocity) is propagated as a Taylor jet of r'' = -mu r / |r|^3 with
 * mu = n^2 a^3, n = 2 pi / p; |r|^-3 is expanded with the power-series rule
 * k q0 s_k = sum_{j=1..k} ((alpha+1) j - k) q_j s_{k-j}, alpha = -3/2. */
void rro_solve2d(double phase, double p, double a, double inc, double e, double w, double *c)
{
    double n = 2.0 * RRO_PI / p;
    double se = sqrt(1.0 - e * e);
    double cth, sth, sf, cf, r;
    if (phase == 0.0) {
        /* conjunction: w + f = pi/2 exactly */
        cth = 0.0; sth = 1.0;
        sf = cos(w); cf = sin(w);
        r = a * (1.0 - e * e) / (1.0 + e * cf);
    } else {
        double f0 = 0.5 * RRO_PI - w;
        double E0 = atan2(se * sin(f0), e + cos(f0));
        double M0 = E0 - e * sin(E0);
        double M = M0 + n * phase;
        double E = rro_ea_newton(M, e);
        double f = atan2(se * sin(E) / (1.0 - e * cos(E)), (cos(E) - e) / (1.0 - e * cos(E)));
        sf = sin(f); cf = cos(f);
        cth = cos(w + f); sth = sin(w + f);
        r = a * (1.0 - e * e) / (1.0 + e * cf);
    }
    double vr = n * a * e * sf / se;          /* dr/dt        */
    double vt = n * a * (1.0 + e * cf) / se;  /* r dtheta/dt  */
    double P[5][2];
    P[0][0] = r * cth;              P[0][1] = r * sth;
    P[1][0] = vr * cth - vt * sth;  P[1][1] = vr * sth + vt * cth;
    double mu = n * n * a * a * a;
    double alpha = -1.5;
    double q0 = P[0][0] * P[0][0] + P[0][1] * P[0][1];
    double q1 = 2.0 * (P[0][0] * P[1][0] + P[0][1] * P[1][1]);
    double s0 = 1.0 / (q0 * sqrt(q0));
    for (int d = 0; d < 2; ++d) P[2][d] = -mu * s0 * P[0][d] / 2.0;
    double s1 = alpha * q1 * s0 / q0;
    for (int d = 0; d < 2; ++d) P[3][d] = -mu * (s0 * P[1][d] + s1 * P[0][d]) / 6.0;
    double q2 = 2.0 * (P[0][0] * P[2][0] + P[0][1] * P[2][1]) + (P[1][0] * P[1][0] + P[1][1] * P[1][1]);
    double s2 = ((alpha - 1.0) * q1 * s1 + 2.0 * alpha * q2 * s0) / (2.0 * q0);
    for (int d = 0; d < 2; ++d) P[4][d] = -mu * (s0 * P[2][d] + s1 * P[1][d] + s2 * P[0][d]) / 12.0;
    double ci = cos(inc);
    for (int j = 0; j < 5; ++j) {
        c[j] = -P[j][0];
        c[5 + j] = -ci * P[j][1];
    }
}

/* Sky position and separation from the Taylor coefficients (sep_c). */
double rro_sep_c(double t, const double *c)
{
    double x = c[0] + t * (c[1] + t * (c[2] + t * (c[3] + t * c[4])));
    double y = c[5] + t * (c[6] + t * (c[7] + t * (c[8] + t * c[9])));
    return sqrt(x * x + y * y);
}

/* Contact-point bisection as pytransit/orbits/taylor_z.py:299-328
 * (initial bracket [0, s*2/|vx|], tolerance 1e-6 d, at most 100 steps), with z
 * from sep_c (time measured from conjunction, no period fold). */
static double rro_contact(double k, int point, const double *c)
{
    double s = (point == 1 || point == 2) ? -1.0 : 1.0;
    double zt = (point == 1 || point == 4) ? 1.0 + k : 1.0 - k;
    double t0 = 0.0;
    double t2 = s * 2.0 / fabs(c[1]);   /* sky speed: dx/dt < 0 about an eclipse */
    double t1 = 0.5 * t2;
    double z0 = rro_sep_c(t0, c) - zt;
    double z1 = rro_sep_c(t1, c) - zt;
    int i = 0;
    while (fabs(t2 - t0) > 1e-6 && i < 100) {
        if (z0 * z1 < 0.0) {
            t2 = t1;
            t1 = 0.5 * (t0 + t1);
            z1 = rro_sep_c(t1, c) - zt;
        } else {
            t0 = t1;
            t1 = 0.5 * (t1 + t2);
            z0 = z1;
            z1 = rro_sep_c(t1, c) - zt;
        }
        i++;
    }
    return t1;
}

void rro_bounding_box(double k, const double *c, double *t1, double *t4)
{
    *t1 = rro_contact(k, 1, c);
    *t4 = rro_contact(k, 4, c);
}

/* Exact-Kepler sky separation (orbits_py.ta_newton_s + z_from_ta_s,
 * orbits_py.py:90-93, 145-154, 192-199): used to measure the Taylor
 * truncation of the orbit layer.  Signed: negative behind the star. */
double rro_z_kepler(double t, double t0, double p, double a, double inc, double e, double w)
{
    double f0 = 0.5 * RRO_PI - w;
    double off = atan2(sqrt(1.0 - e * e) * sin(f0), e + cos(f0));
    off -= e * sin(off);
    double M = fmod(2 * RRO_PI * (t - (t0 - off * p / (2 * RRO_PI))) / p, 2 * RRO_PI);
    if (M < 0) M += 2 * RRO_PI;
    double E = rro_ea_newton(M, e);
    double sta = sqrt(1.0 - e * e) * sin(E) / (1.0 - e * cos(E));
    double cta = (cos(E) - e) / (1.0 - e * cos(E));
    double f = atan2(sta, cta);
    double sw = sin(w + f);
    double z = a * (1.0 - e * e) / (1.0 + e * cos(f)) * sqrt(1.0 - sw * sw * sin(inc) * sin(inc));
    return sw < 0 ? -z : z;
}

/* ------------------------------------------------------------------ */
/* rr_full, pytransit/models/roadrunner/model_full.py:9-100            */
/* ------------------------------------------------------------------ */

/* Limb-darkening means for one parameter vector: the k-lerp of the 3D table
 * (model_full.py:46-51) or a 2D table at k outside [kmin, kmax] or when
 * ik+1 would run past the table (model_full.py:52-55). */
static void rro_ldm_pv(double k0, const double *ldp_pv, int npb, const double *W, int nk, int ng,
                       int nz, double dk, double kmin, double kmax, const double *ze, double *ldm_pv)
{
    int ik = -1;
    double ak = 0.0;
    if (kmin <= k0 && k0 <= kmax) {
        ik = (int)floor((k0 - kmin) / dk);
        ak = (k0 - kmin - ik * dk) / dk;
        if (ik + 1 >= nk) ik = -1;
    }
    if (ik >= 0) {
        const double *W0 = W + (size_t)ik * ng * nz;
        const double *W1 = W0 + (size_t)ng * nz;
        for (int ipb = 0; ipb < npb; ++ipb) {
            const double *l = ldp_pv + (size_t)ipb * nz;
            for (int ig = 0; ig < ng; ++ig) {
                double d0 = 0.0, d1 = 0.0;
                for (int iz = 0; iz < nz; ++iz) {
                    d0 += W0[(size_t)ig * nz + iz] * l[iz];
                    d1 += W1[(size_t)ig * nz + iz] * l[iz];
                }
                ldm_pv[(size_t)ipb * ng + ig] = (1.0 - ak) * d0 + ak * d1;
            }
        }
    } else {
        double *W2 = (double *)malloc(sizeof(double) * ng * nz);
        rro_weights_2d(k0, ze, nz, ng, W2);
        for (int ipb = 0; ipb < npb; ++ipb) {
            const double *l = ldp_pv + (size_t)ipb * nz;
            for (int ig = 0; ig < ng; ++ig) {
                double d = 0.0;
                for (int iz = 0; iz < nz; ++iz) d += W2[(size_t)ig * nz + iz] * l[iz];
                ldm_pv[(size_t)ipb * ng + ig] = d;
            }
        }
        free(W2);
    }
}

/* Full RoadRunner model.  Shapes (row-major, FP64 unless noted):
 *   times[npt], k[npv, nkc] (nkc = 1 or npb), t0[npv, nep], p..w[npv],
 *   lcids[npt] (int32), pbids/epids/nsamples[nlc] (int32), exptimes[nlc],
 *   ldp[npv, npb, nz], istar[npv, npb], W[nk, ng, nz], ze[nz]
 *   -> flux[npv, npt].
 * nthreads <= 0 uses the OpenMP default. Returns 0, or -1 on a bad k shape. */
int rro_rr_full(const double *times, int npt, const double *k, int nkc, const double *t0, int nep,
                const double *p, const double *a, const double *inc, const double *e, const double *w,
                int npv, int nlc, int npb, const int32_t *lcids, const int32_t *pbids,
                const int32_t *epids, const int32_t *nsamples, const double *exptimes,
                const double *ldp, const double *istar, const double *W, int nk, int ng, int nz,
                double dk, double kmin, double kmax, double dg, const double *ze, double *flux,
                int nthreads)
{
    if (nkc > 1 && nkc != npb) return -1;
    double *ks = (double *)malloc(sizeof(double) * (size_t)npv * npb);
    for (int ipv = 0; ipv < npv; ++ipv)
        for (int ipb = 0; ipb < npb; ++ipb)
            ks[(size_t)ipv * npb + ipb] = (nkc == npb) ? k[(size_t)ipv * nkc + ipb] : k[(size_t)ipv * nkc];
    char *good = (char *)malloc(npv);
    double *ldm = (double *)calloc((size_t)npv * npb * ng, sizeof(double));
    double *xyc = (double *)calloc((size_t)npv * 10, sizeof(double));
    double *bbs = (double *)calloc((size_t)npv * nlc * 2, sizeof(double));
#ifdef _OPENMP
    int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif

    #pragma omp parallel for schedule(dynamic, 16) num_threads(nth)
    for (int ipv = 0; ipv < npv; ++ipv) {
        good[ipv] = 1;
        if (isnan(a[ipv]) || a[ipv] <= 1.0 || e[ipv] < 0.0 || isnan(ldp[(size_t)ipv * npb * nz])) {
            good[ipv] = 0;
            continue;
        }
        rro_ldm_pv(ks[(size_t)ipv * npb], ldp + (size_t)ipv * npb * nz, npb, W, nk, ng, nz, dk, kmin,
                   kmax, ze, ldm + (size_t)ipv * npb * ng);
        rro_solve2d(0.0, p[ipv], a[ipv], inc[ipv], e[ipv], w[ipv], xyc + (size_t)ipv * 10);
        double bt1, bt4;
        rro_bounding_box(ks[(size_t)ipv * npb], xyc + (size_t)ipv * 10, &bt1, &bt4);
        for (int ilc = 0; ilc < nlc; ++ilc) {
            bbs[((size_t)ipv * nlc + ilc) * 2 + 0] = bt1 - (0.003 + exptimes[ilc]);
            bbs[((size_t)ipv * nlc + ilc) * 2 + 1] = bt4 + (0.003 + exptimes[ilc]);
        }
    }

    int64_t total = (int64_t)npv * npt;
    #pragma omp parallel for schedule(static) num_threads(nth)
    for (int64_t j = 0; j < total; ++j) {
        int ipv = (int)(j / npt);
        int ipt = (int)(j % npt);
        if (!good[ipv]) { flux[j] = NAN; continue; }
        int ilc = lcids[ipt];
        int ipb = pbids[ilc];
        int iep = epids[ilc];
        double t0v = t0[(size_t)ipv * nep + iep];
        double pv = p[ipv];
        double epoch = floor((times[ipt] - t0v + 0.5 * pv) / pv);
        double tc = times[ipt] - (t0v + epoch * pv);
        const double *bb = bbs + ((size_t)ipv * nlc + ilc) * 2;
        if (!(bb[0] <= tc && tc <= bb[1])) { flux[j] = 1.0; continue; }
        double kk = ks[(size_t)ipv * npb + ipb];
        double is = istar[(size_t)ipv * npb + ipb];
        const double *lda = ldm + ((size_t)ipv * npb + ipb) * ng;
        int ns = nsamples[ilc];
        double f = 0.0;
        for (int isample = 1; isample < ns + 1; ++isample) {
            double toff = exptimes[ilc] * ((isample - 0.5) / ns - 0.5);
            double z = rro_sep_c(tc + toff, xyc + (size_t)ipv * 10);
            double ip = rro_interp_ldm(z / (1.0 + kk), dg, lda, ng);
            double ap = rro_ccia(1.0, kk, z, NULL);
            f += (is - ip * ap) / is;
        }
        flux[j] = f / ns;
    }
    free(ks); free(good); free(ldm); free(xyc); free(bbs);
    return 0;
}

/* ------------------------------------------------------------------ */
/* tsmodel_serial, pytransit/models/roadrunner/model_trspec.py:12-93  */
/* ------------------------------------------------------------------ */

/* Transmission-spectroscopy RoadRunner: k[npv, npb] (one radius ratio per
 * channel), one orbit per pv, LD means at the mean radius ratio, area to
 * first order in k.  Uses only nsamples[0], exptimes[0] and t0[npv] (one
 * epoch), and the 0.0015 d bounding-box pad, as the reference does.
 * weights == NULL selects the per-pv 2D table path.  -> flux[npv, npb, npt] */
int rro_ts_full(const double *times, int npt, const double *k, const double *t0, const double *p,
                const double *a, const double *inc, const double *e, const double *w, int npv,
                int npb, int nsamples0, double exptime0, const double *ldp, const double *istar,
                const double *W, int nk, int ng, int nz, double dk, double kmin, double kmax,
                double dg_in, const double *ze, double *flux, int nthreads)
{
#ifdef _OPENMP
    int nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
    #pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
    for (int ipv = 0; ipv < npv; ++ipv) {
        double *fl = flux + (size_t)ipv * npb * npt;
        if (isnan(a[ipv]) || a[ipv] <= 1.0 || e[ipv] < 0.0) {
            for (size_t j = 0; j < (size_t)npb * npt; ++j) fl[j] = NAN;
            continue;
        }
        for (size_t j = 0; j < (size_t)npb * npt; ++j) fl[j] = 0.0;
        const double *kp = k + (size_t)ipv * npb;
        double kmean = 0.0, kmx = kp[0];
        for (int ipb = 0; ipb < npb; ++ipb) { kmean += kp[ipb]; if (kp[ipb] > kmx) kmx = kp[ipb]; }
        kmean /= npb;
        double *afac = (double *)malloc(sizeof(double) * npb);
        for (int ipb = 0; ipb < npb; ++ipb) afac[ipb] = kp[ipb] * kp[ipb] / (kmean * kmean);
        double *ldm = (double *)malloc(sizeof(double) * npb * ng);
        double dg = dg_in;
        /* model_trspec.py:48: the upper limit is compared against max(k) of this pv */
        if (W != NULL && kmin <= kmean && kmean <= kmx) {
            int ik = (int)floor((kmean - kmin) / dk);
            double ak = (kmean - kmin - ik * dk) / dk;
            const double *W0 = W + (size_t)ik * ng * nz;
            const double *W1 = W0 + (size_t)ng * nz;
            for (int ipb = 0; ipb < npb; ++ipb) {
                const double *l = ldp + ((size_t)ipv * npb + ipb) * nz;
                for (int ig = 0; ig < ng; ++ig) {
                    double d0 = 0.0, d1 = 0.0;
                    for (int iz = 0; iz < nz; ++iz) {
                        d0 += W0[(size_t)ig * nz + iz] * l[iz];
                        d1 += W1[(size_t)ig * nz + iz] * l[iz];
                    }
                    ldm[(size_t)ipb * ng + ig] = (1.0 - ak) * d0 + ak * d1;
                }
            }
        } else {
            double *W2 = (double *)malloc(sizeof(double) * ng * nz);
            dg = rro_weights_2d(kmean, ze, nz, ng, W2);
            for (int ipb = 0; ipb < npb; ++ipb) {
                const double *l = ldp + ((size_t)ipv * npb + ipb) * nz;
                for (int ig = 0; ig < ng; ++ig) {
                    double d = 0.0;
                    for (int iz = 0; iz < nz; ++iz) d += W2[(size_t)ig * nz + iz] * l[iz];
                    ldm[(size_t)ipb * ng + ig] = d;
                }
            }
            free(W2);
        }
        double c[10];
        rro_solve2d(0.0, p[ipv], a[ipv], inc[ipv], e[ipv], w[ipv], c);
        double bt1, bt4;
        rro_bounding_box(kmean, c, &bt1, &bt4);
        bt1 -= 0.0015 + exptime0;
        bt4 += 0.0015 + exptime0;
        for (int ipt = 0; ipt < npt; ++ipt) {
            double epoch = floor((times[ipt] - t0[ipv] + 0.5 * p[ipv]) / p[ipv]);
            double tc = times[ipt] - (t0[ipv] + epoch * p[ipv]);
            if (!(bt1 <= tc && tc <= bt4)) {
                for (int ipb = 0; ipb < npb; ++ipb) fl[(size_t)ipb * npt + ipt] = 1.0;
                continue;
            }
            for (int isample = 1; isample < nsamples0 + 1; ++isample) {
                double toff = exptime0 * ((isample - 0.5) / nsamples0 - 0.5);
                double z = rro_sep_c(tc + toff, c);
                double kappa;
                double ap0 = rro_ccia(1.0, kmean, z, &kappa);
                double dadk = 2.0 * kmean * kappa;
                for (int ipb = 0; ipb < npb; ++ipb) {
                    double is = istar[(size_t)ipv * npb + ipb];
                    double ip = rro_interp_ldm(z / (1.0 + kmean), dg, ldm + (size_t)ipb * ng, ng);
                    double area = (z <= 1.0 - kmx) ? ap0 * afac[ipb] : ap0 + (kp[ipb] - kmean) * dadk;
                    fl[(size_t)ipb * npt + ipt] += (is - ip * area) / is;
                }
            }
            for (int ipb = 0; ipb < npb; ++ipb) fl[(size_t)ipb * npt + ipt] /= nsamples0;
        }
        free(afac);
        free(ldm);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Gaussian log-likelihood, pytransit/lpf/loglikelihood/wnloglikelihood.py:23-35 */
/* ------------------------------------------------------------------ */

/* lnl[ipv] = sum_i -log(sigma) - 0.5 log(2 pi) - 0.5 ((obs_i - model_i)/sigma)^2 */
void rro_lnlike_normal(const double *obs, const double *model, int npv, int npt, double sigma,
                       double *lnl)
{
    for (int ipv = 0; ipv < npv; ++ipv) {
        double s = 0.0;
        for (int i = 0; i < npt; ++i) {
            double r = (obs[i] - model[(size_t)ipv * npt + i]) / sigma;
            s += r * r;
        }
        lnl[ipv] = -npt * log(sigma) - 0.5 * npt * log(2 * RRO_PI) - 0.5 * s;
    }
}

/* ------------------------------------------------------------------ */
/* Mandel & Agol (2002) quadratic model, the independent cross-check:  */
/* eval_quad_z_s, pytransit/models/numba/ma_quadratic_nb.py:277-389     */
/* ------------------------------------------------------------------ */

/* Complete elliptic integral of the first kind, K(k), by the polynomial
 * approximation of Abramowitz & Stegun 17.3.34 in m1 = 1 - k^2
 * (ellk, ma_quadratic_nb.py:110-126). */
double rro_ellk(double k)
{
    double m1 = 1.0 - k * k;
    double ek1 = 1.386294361120 + m1 * (0.096663442590 + m1 * (0.035900923830 + m1 * (0.037425637130 +
                 m1 * 0.014511962120)));
    double ek2 = (0.50 + m1 * (0.124985935970 + m1 * (0.068802485760 + m1 * (0.033283553460 +
                 m1 * 0.004417870120)))) * log(m1);
    return ek1 - ek2;
}

/* Complete elliptic integral of the second kind, E(k), Abramowitz & Stegun
 * 17.3.36 (ellec, ma_quadratic_nb.py:93-107). */
double rro_ellec(double k)
{
    double m1 = 1.0 - k * k;
    double ee1 = 1.0 + m1 * (0.443251414630 + m1 * (0.062606012200 + m1 * (0.047573835460 +
                 m1 * 0.017365064510)));
    double ee2 = m1 * (0.249983683100 + m1 * (0.092001800370 + m1 * (0.040696975260 +
                 m1 * 0.005264496390))) * log(1.0 / m1);
    return ee1 + ee2;
}

/* Complete elliptic integral of the third kind, Pi(n, k), by Bulirsch's
 * (1965) iteration (ellpicb, ma_quadratic_nb.py:55-90); 0 when it does not
 * converge in 1000 steps. */
double rro_ellpicb(double n, double k)
{
    double kc = sqrt(1.0 - k * k), e = kc, p = sqrt(n + 1.0), m0 = 1.0, c = 1.0, d = 1.0 / p;
    for (int it = 0; it < 1000; ++it) {
        double f = c;
        c = d / p + c;
        double g = e / p;
        d = 2.0 * (f * g + d);
        p = g + p;
        g = m0;
        m0 = kc + m0;
        if (fabs(1.0 - kc / g) > 1e-8) {
            kc = 2.0 * sqrt(e);
            e = kc * m0;
        } else {
            return 0.5 * RRO_PI * (c * m0 + d) / (m0 * (m0 + p));
        }
    }
    return 0.0;
}

/* Flux of a star with quadratic limb darkening (u1, u2) occulted by a disk
 * of radius k at centre distance z (Mandel & Agol 2002, Tables 1 and 3), as
 * eval_quad_z_s computes it:
 *   k within 1e-4 of 1/2 is set to 1/2, z within 1e-6 of k is moved by +1e-6;
 *   z > 1 + k or z of negative sign -> 1; k >= 1 and z <= k - 1 -> 0;
 *   the limb angles kap0, kap1 exist only in the ingress/egress branch of
 *   the uniform term; where a later branch reads them without it (z = 1 - k
 *   exactly) they are 0, the value the reference's compiled code uses
 *   (its own test pins F(1 - k) = 0.99164875 for k = 0.1, u = (0.2, 0.1)). */
double rro_ma_quad_z(double z, double k, double u1, double u2)
{
    const double inv_pi = 1.0 / RRO_PI;
    if (fabs(k - 0.5) < 1.0e-4) k = 0.5;
    double k2 = k * k;
    double omega = 1.0 - u1 / 3.0 - u2 / 6.0;
    if (fabs(z - k) < 1e-6) z += 1e-6;
    if (z > 1.0 + k || signbit(z)) return 1.0;
    if (k >= 1.0 && z <= k - 1.0) return 0.0;
    double z2 = z * z, x1 = (k - z) * (k - z), x2 = (k + z) * (k + z), x3 = k * k - z * z;
    double le = 0.0, ld = 0.0, ed = 0.0, kap0 = 0.0, kap1 = 0.0;
    if (z <= 1.0 - k) {
        le = k2;
    } else if (z >= fabs(1.0 - k) && z <= 1.0 + k) {
        kap1 = acos(fmin((1.0 - k2 + z2) / (2.0 * z), 1.0));
        kap0 = acos(fmin((k2 + z2 - 1.0) / (2.0 * k * z), 1.0));
        le = k2 * kap0 + kap1;
        le = (le - 0.5 * sqrt(fmax(4.0 * z2 - (1.0 + z2 - k2) * (1.0 + z2 - k2), 0.0))) * inv_pi;
    }
    int edge_at_origin = fabs(z - k) < 1.e-4 * (z + k);
    int full_transit = k <= 1.0 && z < (1.0 - k);
    if (edge_at_origin) {
        if (k == 0.5) {
            ld = 1.0 / 3.0 - 4.0 * inv_pi / 9.0;
            ed = 3.0 / 32.0;
        } else if (z > 0.5) {
            double q = 0.5 / k, Kk = rro_ellk(q), Ek = rro_ellec(q);
            ld = 1.0 / 3.0 + 16.0 * k / 9.0 * inv_pi * (2.0 * k2 - 1.0) * Ek -
                 (32.0 * k2 * k2 - 20.0 * k2 + 3.0) / 9.0 * inv_pi / k * Kk;
            ed = 0.5 * inv_pi * (kap1 + k2 * (k2 + 2.0 * z2) * kap0 -
                                 (1.0 + 5.0 * k2 + z2) / 4.0 * sqrt((1.0 - x1) * (x2 - 1.0)));
        } else if (z < 0.5) {
            double q = 2.0 * k, Kk = rro_ellk(q), Ek = rro_ellec(q);
            ld = 1.0 / 3.0 + 2.0 / 9.0 * inv_pi * (4.0 * (2.0 * k2 - 1.0) * Ek + (1.0 - 4.0 * k2) * Kk);
            ed = k2 / 2.0 * (k2 + 2.0 * z2);
        }
    } else if (full_transit) {
        double q = sqrt((x2 - x1) / (1.0 - x1)), Kk = rro_ellk(q), Ek = rro_ellec(q);
        double Pk = rro_ellpicb(x2 / x1 - 1.0, q);
        ld = 2.0 / 9.0 * inv_pi / sqrt(1.0 - x1) *
             ((1.0 - 5.0 * z2 + k2 + x3 * x3) * Kk + (1.0 - x1) * (z2 + 7.0 * k2 - 4.0) * Ek - 3.0 * x3 / x1 * Pk);
        if (z < k) ld = ld + 2.0 / 3.0;
        if (fabs(k + z - 1.0) < 1.e-4)
            ld = 2.0 / 3.0 * inv_pi * acos(1.0 - 2.0 * k) - 4.0 / 9.0 * inv_pi * sqrt(k * (1.0 - k)) *
                 (3.0 + 2.0 * k - 8.0 * k2);
        ed = k2 / 2.0 * (k2 + 2.0 * z2);
    } else {
        double q = sqrt((1.0 - (k - z) * (k - z)) / 4.0 / z / k), Kk = rro_ellk(q), Ek = rro_ellec(q);
        double Pk = rro_ellpicb(1.0 / x1 - 1.0, q);
        ld = 1.0 / 9.0 * inv_pi / sqrt(k * z) *
             (((1.0 - x2) * (2.0 * x2 + x1 - 3.0) - 3.0 * x3 * (x2 - 2.0)) * Kk +
              4.0 * k * z * (z2 + 7.0 * k2 - 4.0) * Ek - 3.0 * x3 / x1 * Pk);
        if (z < k) ld = ld + 2.0 / 3.0;
        ed = 0.5 * inv_pi * (kap1 + k2 * (k2 + 2.0 * z2) * kap0 -
                             (1.0 + 5.0 * k2 + z2) / 4.0 * sqrt((1.0 - x1) * (x2 - 1.0)));
    }
    return 1.0 - ((1.0 - u1 - 2.0 * u2) * le + (u1 + 2.0 * u2) * ld + u2 * ed) / omega;
}

/* rro_ma_quad_z over an array of z. */
void rro_ma_quad_z_v(const double *z, int n, double k, double u1, double u2, double *flux)
{
    for (int i = 0; i < n; ++i) flux[i] = rro_ma_quad_z(z[i], k, u1, u2);
}

/* ------------------------------------------------------------------ */
/* RoadRunner secondary eclipse: eclipse_model (model_eclipse.py:12-81) */
/* and the spectroscopic esmodel (model_ecspec.py:13-63)               */
/* ------------------------------------------------------------------ */

/* Time from mid-transit to mid-eclipse (meepmeep's eclipse_time_offset, not
 * in the reference; restated as the reference's own eclipse_phase,
 * pytransit/orbits/orbits_py.py:544-555): from the mean anomalies at the two
 * conjunctions, wrapped to (0, p]. */
double rro_eclipse_time_offset(double p, double inc, double e, double w)
{
    (void)inc;
    double se = sqrt(1.0 - e * e);
    double etr = atan2(se * sin(0.5 * RRO_PI - w), e + cos(0.5 * RRO_PI - w));
    double eec = atan2(se * sin(0.5 * RRO_PI + RRO_PI - w), e + cos(0.5 * RRO_PI + RRO_PI - w));
    double mtr = etr - e * sin(etr), mec = eec - e * sin(eec);
    double ph = (mec - mtr) * p / (2.0 * RRO_PI);
    return ph > 0.0 ? ph : p + ph;
}

/* Light travel time of the eclipse relative to the transit in days (meepmeep's
 * eclipse_light_travel_time, not in the reference; restated from the
 * geometry): (r_transit + r_eclipse) sin i stellar radii of rstar solar radii
 * (IAU nominal 6.957e8 m) over c. */
double rro_eclipse_ltt(double p, double a, double inc, double e, double w, double rstar)
{
    (void)p;
    double r_tr = a * (1.0 - e * e) / (1.0 + e * cos(0.5 * RRO_PI - w));
    double r_ec = a * (1.0 - e * e) / (1.0 + e * cos(1.5 * RRO_PI - w));
    return (r_tr + r_ec) * sin(inc) * rstar * 6.957e8 / 299792458.0 / 86400.0;
}

/* eclipse_model: the visible area of the planet disk, pi k^2 outside the
 * eclipse bounding box (padded by 0.003 d + exptime), else the mean over the
 * exposure samples of pi k^2 - A(1, k, z), z from the Taylor series about
 * mid-eclipse; t0[npv, nep] per epoch; NaN rows for a NaN or <= 1, e < 0. */
void rro_eclipse_full(const double *times, int npt, const double *k, const double *t0, int nep, const double *p,
                      const double *a, const double *inc, const double *e, const double *w, int npv, double rstar,
                      int nlc, const int32_t *lcids, const int32_t *epids, const int32_t *nsamples,
                      const double *exptimes, double *flux)
{
    #pragma omp parallel for schedule(dynamic, 1)
    for (int ipv = 0; ipv < npv; ++ipv) {
        double *fl = flux + (size_t)ipv * npt;
        if (isnan(a[ipv]) || a[ipv] <= 1.0 || e[ipv] < 0.0) {
            for (int j = 0; j < npt; ++j) fl[j] = NAN;
            continue;
        }
        double shift = rro_eclipse_time_offset(p[ipv], inc[ipv], e[ipv], w[ipv]);
        double c[10];
        rro_solve2d(shift, p[ipv], a[ipv], inc[ipv], e[ipv], w[ipv], c);
        double ltt = rro_eclipse_ltt(p[ipv], a[ipv], inc[ipv], e[ipv], w[ipv], rstar);
        double bt1, bt4;
        rro_bounding_box(k[ipv], c, &bt1, &bt4);
        double pik2 = RRO_PI * (k[ipv] * k[ipv]);
        for (int j = 0; j < npt; ++j) {
            int ilc = lcids[j];
            double te = t0[(size_t)ipv * nep + epids[ilc]] + shift + ltt;
            double epoch = floor((times[j] - te + 0.5 * p[ipv]) / p[ipv]);
            double tc = times[j] - (te + epoch * p[ipv]);
            double lo = bt1 - (0.003 + exptimes[ilc]), hi = bt4 + (0.003 + exptimes[ilc]);
            (void)nlc;
            if (!(lo <= tc && tc <= hi)) {
                fl[j] = pik2;
            } else {
                double f = 0.0;
                int ns = nsamples[ilc];
                for (int is = 1; is < ns + 1; ++is) {
                    double toff = exptimes[ilc] * ((is - 0.5) / ns - 0.5);
                    double z = rro_sep_c(tc + toff, c), kap;
                    f += pik2 - rro_ccia(1.0, k[ipv], z, &kap);
                }
                fl[j] = f / ns;
            }
        }
    }
}

/* esmodel: flux[npv, npb, npt] = 1 outside the box (padded by 0.0015 d +
 * exptime), else the mean over the samples of
 * 1 - (f_b A(1, k, z) / pi) / (1 + f_b k^2); one zero epoch t0[npv], the
 * first light curve's nsamples and exptime, rstar[npv]. */
void rro_es_full(const double *times, int npt, const double *k, const double *t0, const double *p, const double *a,
                 const double *inc, const double *e, const double *w, const double *rstar, const double *fratio,
                 int npv, int npb, int nsamples, double exptime, double *flux)
{
    #pragma omp parallel for schedule(dynamic, 1)
    for (int ipv = 0; ipv < npv; ++ipv) {
        double *fl = flux + (size_t)ipv * npb * npt;
        if (isnan(a[ipv]) || a[ipv] <= 1.0 || e[ipv] < 0.0) {
            for (size_t j = 0; j < (size_t)npb * npt; ++j) fl[j] = NAN;
            continue;
        }
        double shift = rro_eclipse_time_offset(p[ipv], inc[ipv], e[ipv], w[ipv]);
        double c[10];
        rro_solve2d(shift, p[ipv], a[ipv], inc[ipv], e[ipv], w[ipv], c);
        double ltt = rro_eclipse_ltt(p[ipv], a[ipv], inc[ipv], e[ipv], w[ipv], rstar[ipv]);
        double te = t0[ipv] + shift + ltt;
        double bt1, bt4;
        rro_bounding_box(k[ipv], c, &bt1, &bt4);
        bt1 -= 0.0015 + exptime;
        bt4 += 0.0015 + exptime;
        for (int j = 0; j < npt; ++j) {
            double epoch = floor((times[j] - te + 0.5 * p[ipv]) / p[ipv]);
            double tc = times[j] - (te + epoch * p[ipv]);
            if (!(bt1 <= tc && tc <= bt4)) {
                for (int b = 0; b < npb; ++b) fl[(size_t)b * npt + j] = 1.0;
                continue;
            }
            for (int b = 0; b < npb; ++b) fl[(size_t)b * npt + j] = 0.0;
            for (int is = 1; is < nsamples + 1; ++is) {
                double toff = exptime * ((is - 0.5) / nsamples - 0.5);
                double z = rro_sep_c(tc + toff, c), kap;
                double ar = rro_ccia(1.0, k[ipv], z, &kap);
                for (int b = 0; b < npb; ++b) {
                    double f = fratio[(size_t)ipv * npb + b];
                    fl[(size_t)b * npt + j] += 1.0 - (f * ar / RRO_PI) / (1.0 + f * (k[ipv] * k[ipv]));
                }
            }
            for (int b = 0; b < npb; ++b) fl[(size_t)b * npt + j] /= nsamples;
        }
    }
}
