/*
 * ORACLE (test infrastructure only) -- literal closed-shell "r-ccsd" of helios.
 *
 * A term-by-term C restatement of the reference's spatial-orbital RHF-CCSD,
 * used to pin the GPU path and as the timed CPU baseline of the reference
 * algorithm. Nothing in the product links this file.
 *
 *   integrals  R(a,b,c,d) = 2(ab|cd) - (ad|cb), ZDO form
 *              src/methods/coupledCluster/mod_cc.f90:2258-2277 (filled :547-557)
 *   guess      mod_cc.f90:634-650
 *   singles    src/methods/coupledCluster/ccsd/proj-ccsd-spat-hf-1.f90:14-119
 *   doubles    src/methods/coupledCluster/ccsd/proj-ccsd-spat-hf-2.f90:14-256
 *   step       mod_cc.f90:987-1017 (projection types "1" and "2-1")
 *   DIIS       pushCCVectors mod_cc.f90:1390-1423, newCCVectors :1514-1555,1643-1671,
 *              diisDotProduct :2133-2193
 *   energy     energyCC mod_cc.f90:1916-1952
 *   loop       iterationCC mod_cc.f90:820-891 + gIterator.f90:88-210 stop rules
 *
 * Layout (0-based, row-major): orbital indices p in [0,N), occupied i<o,
 * virtual a in [o,N). F[p*N+q]; R[((p*N+q)*N+r)*N+s]; C[mu*N+p] (site mu,
 * MO p); t1[i*v+(a-o)]; t2[((i*o+j)*v+(a-o))*v+(b-o)]. The excitation list is
 * the reference's: mm = i*v + (a-o), i outer, a inner; pairs mm <= nn.
 *
 * The reference opens an OpenMP reduction around every inner sum; here the
 * outer pair loop is parallel and every inner sum runs sequentially, so a run
 * is deterministic for any thread count.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RR(p, q, r, s) R[(((size_t)(p) * N + (q)) * N + (r)) * N + (s)]
#define FF(p, q) F[(size_t)(p) * N + (q)]
#define T1(i, a) t1[(size_t)(i) * v + ((a) - o)]
#define T2(i, j, a, b) t2[(((size_t)(i) * o + (j)) * v + ((a) - o)) * v + ((b) - o)]
#define D2(i, j, a, b) d2[(((size_t)(i) * o + (j)) * v + ((a) - o)) * v + ((b) - o)]

/* R(a,b,c,d) = sum_{mu,nu} (2 C_mu,a C_mu,b C_nu,d - C_mu,a C_mu,d C_nu,b) C_nu,c G_mu,nu */
void orc_integrals(int N, const double *C, const double *G, double *R)
{
    #pragma omp parallel for collapse(2) schedule(static)
    for (int a = 0; a < N; ++a)
        for (int b = 0; b < N; ++b)
            for (int c = 0; c < N; ++c)
                for (int d = 0; d < N; ++d) {
                    double sum = 0.0;
                    for (int mu = 0; mu < N; ++mu) {
                        double ir1 = 2.0 * C[mu * N + a] * C[mu * N + b];
                        double ir2 = C[mu * N + a] * C[mu * N + d];
                        for (int nu = 0; nu < N; ++nu) {
                            double irt = (ir1 * C[nu * N + d] - ir2 * C[nu * N + b]) * C[nu * N + c];
                            sum += irt * G[mu * N + nu];
                        }
                    }
                    RR(a, b, c, d) = sum;
                }
}

void orc_guess(int N, int o, const double *F, const double *R, double *t1, double *t2)
{
    int v = N - o, ne = o * v;
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        T1(i, a) = FF(i, a) / (FF(i, i) - FF(a, a));
        for (int nn = mm; nn < ne; ++nn) {
            int j = nn / v, b = o + nn % v;
            T2(i, j, a, b) = RR(i, a, j, b) / (FF(i, i) + FF(j, j) - FF(a, a) - FF(b, b));
            T2(j, i, b, a) = T2(i, j, a, b);
        }
    }
}

void orc_singles(int N, int o, const double *F, const double *R,
                 const double *t1, const double *t2, double *d1)
{
    int v = N - o, ne = o * v;
    #pragma omp parallel for schedule(dynamic)
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        double rez = FF(i, a), sum;                         /* 6 */
        sum = 0;                                            /* 8 */
        for (int j = 0; j < o; ++j)
            for (int b = o; b < N; ++b) sum += RR(a, i, j, b) * T1(j, b);
        rez += sum;
        sum = 0;                                            /* 7 */
        for (int b = o; b < N; ++b) sum += FF(a, b) * T1(i, b);
        rez += sum;
        sum = 0;                                            /* 7 */
        for (int j = 0; j < o; ++j) sum += FF(i, j) * T1(j, a);
        rez -= sum;
        sum = 0;                                            /* 9 */
        for (int j = 0; j < o; ++j)
            for (int b = o; b < N; ++b) sum += FF(j, b) * (2 * T2(i, j, a, b) - T2(j, i, a, b));
        rez += sum;
        sum = 0;                                            /* 10 */
        for (int j = 0; j < o; ++j)
            for (int b = o; b < N; ++b)
                for (int c = o; c < N; ++c)
                    sum += RR(a, b, j, c) * (T2(i, j, b, c) + T1(i, b) * T1(j, c));
        rez += sum;
        sum = 0;                                            /* 11 */
        for (int j = 0; j < o; ++j)
            for (int k = 0; k < o; ++k)
                for (int b = o; b < N; ++b)
                    sum += RR(k, b, j, i) * (T2(j, k, a, b) + T1(j, a) * T1(k, b));
        rez -= sum;
        sum = 0;                                            /* 12 */
        for (int j = 0; j < o; ++j)
            for (int b = o; b < N; ++b) sum += FF(j, b) * T1(i, b) * T1(j, a);
        rez -= sum;
        sum = 0;                                            /* 13 */
        for (int j = 0; j < o; ++j)
            for (int k = 0; k < o; ++k)
                for (int b = o; b < N; ++b)
                    for (int c = o; c < N; ++c)
                        sum += RR(k, c, j, b) * (+T1(k, c) * (2 * T2(i, j, a, b) - T2(j, i, a, b))
                                                 - T1(i, b) * T2(j, k, a, c)
                                                 - T1(k, a) * (T2(j, i, b, c) + T1(j, b) * T1(i, c)));
        rez += sum;
        d1[(size_t)i * v + (a - o)] = rez;
    }
}

/* The doubles formula for one pair of excitations (i,a), (j,b). */
static double doubles_pair(int N, int o, const double *F, const double *R, const double *t1, const double *t2,
                           int i, int a, int j, int b)
{
    int v = N - o;
    {
        {
            double rez = RR(a, i, b, j), sum;               /* 14 */

            sum = 0;                                        /* 25 */
            for (int c = o; c < N; ++c)
                sum += RR(b, j, a, c) * T1(i, c) + RR(a, i, b, c) * T1(j, c);
            rez += sum;

            sum = 0;                                        /* 26 */
            for (int k = 0; k < o; ++k)
                sum += RR(k, i, b, j) * T1(k, a) + RR(k, j, a, i) * T1(k, b);
            rez -= sum;

            sum = 0;                                        /* 17 */
            for (int k = 0; k < o; ++k)
                for (int l = 0; l < o; ++l)
                    sum += RR(k, i, l, j) * (T2(k, l, a, b) + T1(k, a) * T1(l, b));
            rez += sum;

            sum = 0;                                        /* 18 */
            for (int c = o; c < N; ++c)
                for (int d = o; d < N; ++d)
                    sum += RR(b, d, a, c) * (T2(i, j, c, d) + T1(i, c) * T1(j, d));
            rez += sum;

            sum = 0;                                        /* 19-22, 27, 28 */
            for (int k = 0; k < o; ++k)
                for (int c = o; c < N; ++c) {
                    sum += 2 * (+T2(i, k, a, c) * RR(b, j, k, c)
                                + T2(j, k, b, c) * RR(a, i, k, c)
                                + (-T2(i, k, c, a) * RR(k, c, b, j)
                                   - T2(j, k, c, b) * RR(k, c, a, i)
                                   - T2(j, k, a, c) * RR(k, c, b, i)
                                   - T2(i, k, b, c) * RR(k, c, a, j)
                                   - T2(k, j, a, c) * RR(k, i, b, c)
                                   - T2(k, i, b, c) * RR(k, j, a, c)) / 2);
                    sum += (-RR(a, c, k, j) * T1(i, c) * T1(k, b)
                            - RR(b, c, k, i) * T1(j, c) * T1(k, a)
                            - RR(k, c, b, j) * T1(i, c) * T1(k, a)
                            - RR(k, c, a, i) * T1(j, c) * T1(k, b));
                }
            rez += sum;

            sum = 0;                                        /* 33, 36, 38 */
            for (int k = 0; k < o; ++k)
                for (int c = o; c < N; ++c)
                    for (int d = o; d < N; ++d) {
                        sum += RR(k, c, b, d) * (T1(j, d) * (2 * T2(i, k, a, c) - T2(k, i, a, c))
                                                 - T2(j, k, a, c) * T1(i, d)
                                                 - T2(k, j, a, d) * T1(i, c))
                             + RR(k, c, a, d) * (T1(i, d) * (2 * T2(j, k, b, c) - T2(k, j, b, c))
                                                 - T2(i, k, b, c) * T1(j, d)
                                                 - T2(k, i, b, d) * T1(j, c));
                        sum += T1(k, d) * (RR(k, d, b, c) * (2 * T2(i, j, a, c) - T2(i, j, c, a))
                                           + RR(k, d, a, c) * (2 * T2(j, i, b, c) - T2(j, i, c, b)));
                        sum += -RR(a, c, k, d) * T1(k, b) * (T2(i, j, c, d) + T1(i, c) * T1(j, d))
                               - RR(b, c, k, d) * T1(k, a) * (T2(j, i, c, d) + T1(j, c) * T1(i, d));
                    }
            rez += sum;

            sum = 0;                                        /* 34, 35, 37 */
            for (int k = 0; k < o; ++k)
                for (int c = o; c < N; ++c)
                    for (int l = 0; l < o; ++l) {
                        sum += RR(k, c, l, j) * (T1(l, b) * (-2 * T2(i, k, a, c) + T2(k, i, a, c))
                                                 + T2(i, k, b, c) * T1(l, a)
                                                 + T2(i, l, c, b) * T1(k, a))
                             + RR(k, c, l, i) * (T1(l, a) * (-2 * T2(j, k, b, c) + T2(k, j, b, c))
                                                 + T2(j, k, a, c) * T1(l, b)
                                                 + T2(j, l, c, a) * T1(k, b));
                        sum += T1(l, c) * (RR(k, j, l, c) * (-2 * T2(i, k, a, b) + T2(k, i, a, b))
                                           + RR(k, i, l, c) * (-2 * T2(j, k, b, a) + T2(k, j, b, a)));
                        sum += RR(k, c, l, j) * T1(i, c) * (T2(k, l, a, b) + T1(k, a) * T1(l, b))
                             + RR(k, c, l, i) * T1(j, c) * (T2(k, l, b, a) + T1(k, b) * T1(l, a));
                    }
            rez += sum;

            sum = 0;                                        /* 23, 24, 39 */
            for (int k = 0; k < o; ++k)
                for (int c = o; c < N; ++c)
                    for (int l = 0; l < o; ++l)
                        for (int d = o; d < N; ++d) {
                            sum += RR(k, c, l, d) * (
                                -2 * (T2(l, j, d, b) * T1(i, c) * T1(k, a) + T2(l, i, d, a) * T1(j, c) * T1(k, b)
                                      + T2(l, j, a, b) * T1(k, c) * T1(i, d) + T2(l, i, b, a) * T1(k, c) * T1(j, d)
                                      + T2(i, j, a, c) * T1(k, b) * T1(l, d) + T2(j, i, b, c) * T1(k, a) * T1(l, d)
                                      + T2(k, i, c, d) * T2(l, j, a, b) + T2(k, j, c, d) * T2(l, i, b, a)
                                      + T2(i, j, a, c) * T2(k, l, b, d) + T2(j, i, b, c) * T2(k, l, a, d)
                                      + T2(i, k, c, a) * T2(l, j, d, b) + T2(j, k, c, b) * T2(l, i, d, a)
                                      - T2(i, k, a, c) * T2(l, j, d, b) - T2(j, k, b, c) * T2(l, i, d, a))
                                + T2(j, l, d, b) * T1(i, c) * T1(k, a) + T2(i, l, d, a) * T1(j, c) * T1(k, b)
                                + T2(l, i, d, b) * T1(j, c) * T1(k, a) + T2(l, j, d, a) * T1(i, c) * T1(k, b)
                                + T2(i, l, c, b) * T1(j, d) * T1(k, a) + T2(j, l, c, a) * T1(i, d) * T1(k, b)
                                + T2(l, i, a, b) * T1(k, c) * T1(j, d) + T2(l, j, b, a) * T1(k, c) * T1(i, d)
                                + T2(i, j, c, a) * T1(k, b) * T1(l, d) + T2(j, i, c, b) * T1(k, a) * T1(l, d)
                                + T2(k, l, a, b) * T1(i, c) * T1(j, d)
                                + T2(i, j, c, d) * (T2(k, l, a, b) + T1(k, a) * T1(l, b))
                                + T1(i, c) * T1(k, a) * T1(j, d) * T1(l, b)
                                + T2(k, j, c, d) * T2(l, i, a, b) + T2(k, i, c, d) * T2(l, j, b, a)
                                + T2(i, j, b, c) * T2(k, l, a, d) + T2(j, i, a, c) * T2(k, l, b, d)
                                - T2(l, i, d, b) * (T2(j, k, a, c) - T2(j, k, c, a))
                                - T2(l, j, d, a) * (T2(i, k, b, c) - T2(i, k, c, b))
                                + (T2(i, k, c, a) * T2(j, l, d, b) + T2(j, k, c, b) * T2(i, l, d, a)
                                   + T2(j, k, d, a) * T2(i, l, c, b) + T2(i, k, d, b) * T2(j, l, c, a)) / 2);
                        }
            rez += sum;

            sum = 0;                                        /* 15 */
            for (int c = o; c < N; ++c)
                sum += FF(c, a) * (2 * T2(i, j, c, b) - T2(j, i, c, b))
                     + FF(c, b) * (2 * T2(j, i, c, a) - T2(i, j, c, a));
            rez += sum;

            sum = 0;                                        /* 16 */
            for (int k = 0; k < o; ++k)
                sum += FF(k, i) * (2 * T2(k, j, a, b) - T2(k, j, b, a))
                     + FF(k, j) * (2 * T2(k, i, b, a) - T2(k, i, a, b));
            rez -= sum;

            sum = 0;                                        /* 29-32 */
            for (int k = 0; k < o; ++k)
                for (int c = o; c < N; ++c)
                    sum += FF(k, c) * (-2 * (+T2(k, j, a, b) * T1(i, c) + T2(k, i, b, a) * T1(j, c)
                                             + T2(i, j, a, c) * T1(k, b) + T2(j, i, b, c) * T1(k, a))
                                       + T2(k, i, a, b) * T1(j, c) + T2(k, j, b, a) * T1(i, c)
                                       + T2(j, i, a, c) * T1(k, b) + T2(i, j, b, c) * T1(k, a));
            rez += sum;

            return rez;
        }
    }
}

void orc_doubles(int N, int o, const double *F, const double *R,
                 const double *t1, const double *t2, double *d2)
{
    int v = N - o, ne = o * v;
    #pragma omp parallel for schedule(dynamic)
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        for (int nn = mm; nn < ne; ++nn) {
            int j = nn / v, b = o + nn % v;
            double rez = doubles_pair(N, o, F, R, t1, t2, i, a, j, b);
            D2(i, j, a, b) = rez;
            D2(j, i, b, a) = rez;
        }
    }
}

/* The doubles formula on a list of pairs (mm[k], nn[k]) only: a bounded
 * sample of one reference iteration, for timing on large systems. */
void orc_doubles_sample(int N, int o, const double *F, const double *R, const double *t1, const double *t2,
                        const int *mm, const int *nn, int npairs, double *out)
{
    int v = N - o;
    #pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < npairs; ++k) {
        int i = mm[k] / v, a = o + mm[k] % v, j = nn[k] / v, b = o + nn[k] % v;
        out[k] = doubles_pair(N, o, F, R, t1, t2, i, a, j, b);
    }
}

/* stepCC r-ccsd (mod_cc.f90:987-1017); acc[0]=max|d1|, acc[1]=max|d2| */
void orc_step(int N, int o, const double *F, double *t1, double *t2,
              const double *d1, const double *d2, double step1, double step2,
              int projtype, double *acc)
{
    int v = N - o, ne = o * v;
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        T1(i, a) = T1(i, a) + step1 * d1[(size_t)i * v + (a - o)] / (FF(i, i) - FF(a, a));
    }
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        for (int nn = mm; nn < ne; ++nn) {
            int j = nn / v, b = o + nn % v;
            double den = FF(i, i) - FF(a, a) + FF(j, j) - FF(b, b);
            if (projtype == 1)
                T2(i, j, a, b) = T2(i, j, a, b) + step2 * D2(i, j, a, b) / den;
            else
                T2(i, j, a, b) = T2(i, j, a, b) + step2 * (2 * D2(i, j, a, b) + D2(i, j, b, a)) / den;
            T2(j, i, b, a) = T2(i, j, a, b);
        }
    }
    double m1 = 0, m2 = 0;
    for (size_t x = 0; x < (size_t)ne; ++x) m1 = fmax(m1, fabs(d1[x]));
    for (size_t x = 0; x < (size_t)ne * ne; ++x) m2 = fmax(m2, fabs(d2[x]));
    acc[0] = m1; acc[1] = m2;
}

/* energyCC r-ccsd (mod_cc.f90:1916-1952); e[0..3] = total, Eref, 2*sum1, 2*sum2+sum3 */
void orc_energy(int N, int o, const double *F, const double *R, const double *t1,
                const double *t2, double eref, double *e)
{
    int v = N - o, ne = o * v;
    double s1 = 0, s2 = 0, s3 = 0;
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        s1 += FF(i, a) * T1(i, a);
    }
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        for (int nn = mm + 1; nn < ne; ++nn) {
            int j = nn / v, b = o + nn % v;
            s2 += RR(a, i, b, j) * (T2(i, j, a, b) + T1(i, a) * T1(j, b));
        }
    }
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        s3 += RR(a, i, a, i) * (T2(i, i, a, a) + T1(i, a) * T1(i, a));
    }
    e[0] = 2 * s1 + (2 * s2 + s3) + eref;
    e[1] = eref;
    e[2] = 2 * s1;
    e[3] = 2 * s2 + s3;
    e[4] = 0;
}

/* Cyclic Jacobi eigen-decomposition of a small symmetric n x n matrix (row-major).
 * Any FP64 symmetric eigensolver serves the DIIS solve of newCCVectors. */
static void jacobi_eig(int n, double *A, double *V, double *w)
{
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) V[i * n + j] = (i == j);
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
        if (off < 1e-300) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = A[p * n + q];
                if (fabs(apq) < 1e-300) continue;
                double theta = (A[q * n + q] - A[p * n + p]) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = A[i * n + i];
}

/* DIIS state: history slots 0..nd-1 (slot 0 newest), packed singles (ne) and
 * doubles over pairs mm<=nn (ne(ne+1)/2), bordered Gram matrix (nd+1)^2. */
typedef struct {
    int nd, ne;
    size_t np;
    double *sd1, *st1, *sd2, *st2, *B;
} diis_t;

static void diis_push(diis_t *h, int N, int o, const double *t1, const double *t2,
                      const double *d1, const double *d2, int projtype)
{
    int v = N - o, ne = o * v;
    for (int k = h->nd - 1; k >= 1; --k) {
        memcpy(h->sd1 + (size_t)k * ne, h->sd1 + (size_t)(k - 1) * ne, sizeof(double) * ne);
        memcpy(h->st1 + (size_t)k * ne, h->st1 + (size_t)(k - 1) * ne, sizeof(double) * ne);
        memcpy(h->sd2 + (size_t)k * h->np, h->sd2 + (size_t)(k - 1) * h->np, sizeof(double) * h->np);
        memcpy(h->st2 + (size_t)k * h->np, h->st2 + (size_t)(k - 1) * h->np, sizeof(double) * h->np);
    }
    for (int mm = 0; mm < ne; ++mm) { h->sd1[mm] = d1[mm]; h->st1[mm] = t1[mm]; }
    size_t vv = 0;
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        for (int nn = mm; nn < ne; ++nn, ++vv) {
            int j = nn / v, b = o + nn % v;
            h->st2[vv] = T2(i, j, a, b);
            h->sd2[vv] = projtype == 1 ? D2(i, j, a, b) : 2 * D2(i, j, a, b) + D2(i, j, b, a);
        }
    }
}

/* Gaussian elimination with partial pivoting; solves A x = b in place (x -> b). */
static void gauss_solve(int n, double *A, double *b)
{
    for (int k = 0; k < n; ++k) {
        int piv = k;
        for (int r = k + 1; r < n; ++r)
            if (fabs(A[r * n + k]) > fabs(A[piv * n + k])) piv = r;
        if (piv != k) {
            for (int c = 0; c < n; ++c) { double t = A[k * n + c]; A[k * n + c] = A[piv * n + c]; A[piv * n + c] = t; }
            double t = b[k]; b[k] = b[piv]; b[piv] = t;
        }
        for (int r = k + 1; r < n; ++r) {
            double f = A[r * n + k] / A[k * n + k];
            for (int c = k; c < n; ++c) A[r * n + c] -= f * A[k * n + c];
            b[r] -= f * b[k];
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        double s = b[k];
        for (int c = k + 1; c < n; ++c) s -= A[k * n + c] * b[c];
        b[k] = s / A[k * n + k];
    }
}

/* solver 0: Gaussian elimination (default); solver 1: the reference's route,
 * c_k = sum_l V(k,l) V(ub,l) / lambda_l from an eigen-decomposition of the
 * bordered matrix. Both give B^-1 e_ub in exact arithmetic; the eigen route
 * loses the smallest Gram eigenvalues to rounding once residuals fall to
 * ~1e-9 and then stalls. */
static void diis_new(diis_t *h, int N, int o, int iteration, double *t1, double *t2, int solver)
{
    int v = N - o, ne = o * v, ld = h->nd + 1;
    double *B = h->B;
    for (int k = iteration - 1; k >= 1; --k)
        for (int l = iteration - 1; l >= 1; --l) B[k * ld + l] = B[(k - 1) * ld + (l - 1)];
    for (int k = 0; k < iteration; ++k) {
        double s1 = 0, s2 = 0;
        for (int x = 0; x < ne; ++x) s1 += h->sd1[(size_t)k * ne + x] * h->sd1[x];
        for (size_t x = 0; x < h->np; ++x) s2 += h->sd2[(size_t)k * h->np + x] * h->sd2[x];
        B[k * ld + 0] = B[0 * ld + k] = s1 + s2;
    }
    if (iteration == 1) return;
    int ub = iteration; /* 0-based index of the border row */
    for (int k = 0; k <= ub; ++k) { B[k * ld + ub] = 1; B[ub * ld + k] = 1; }
    B[ub * ld + ub] = 0;
    int n = ub + 1;
    double *A = malloc(sizeof(double) * n * n), *V = malloc(sizeof(double) * n * n),
           *w = malloc(sizeof(double) * n), *c = malloc(sizeof(double) * n);
    for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q) A[p * n + q] = B[p * ld + q];
    if (solver == 1) {
        jacobi_eig(n, A, V, w);
        for (int k = 0; k < iteration; ++k) {
            c[k] = 0;
            for (int l = 0; l < n; ++l) c[k] += V[k * n + l] * V[ub * n + l] / w[l];
        }
    } else {
        for (int k = 0; k < n; ++k) c[k] = (k == ub);
        gauss_solve(n, A, c);
    }
    /* a singular subspace (more vectors than the amplitude space has
     * dimensions) gives no usable mixing: keep the stepped amplitudes */
    for (int k = 0; k < iteration; ++k)
        if (!isfinite(c[k])) { free(A); free(V); free(w); free(c); return; }
    for (int x = 0; x < ne; ++x) {
        double s = 0;
        for (int p = 0; p < iteration; ++p) s += c[p] * h->st1[(size_t)p * ne + x];
        t1[x] = s;
    }
    size_t vv = 0;
    for (int mm = 0; mm < ne; ++mm) {
        int i = mm / v, a = o + mm % v;
        for (int nn = mm; nn < ne; ++nn, ++vv) {
            int j = nn / v, b = o + nn % v;
            double s = 0;
            for (int p = 0; p < iteration; ++p) s += c[p] * h->st2[(size_t)p * h->np + vv];
            T2(i, j, a, b) = s;
            T2(j, i, b, a) = s;
        }
    }
    free(A); free(V); free(w); free(c);
}

/*
 * Full r-ccsd solve: iterationCC + energyCC under the gIterator stop rules.
 * t1/t2 must hold the starting amplitudes (orc_guess, or a caller guess).
 * params: step1, step2, eps, divergence, stagnation_pct
 * iparams: maxiter, diis_on, nd, projtype, stagnation_after, check_div, check_stag,
 *          diis_solver (0 Gaussian elimination, 1 eigen-decomposition)
 * trace (optional, 3 doubles per iteration): max|d1|, max|d2|, E_total.
 * Returns the status (1 converged, -1 maxiter, -2 diverged, -3 stagnated).
 */
int orc_ccsd_solve(int N, int o, const double *F, const double *R, double eref,
                   double *t1, double *t2, const double *params, const int *iparams,
                   double *energy, int *iterations, double *trace, int trace_cap)
{
    int v = N - o, ne = o * v;
    double step1 = params[0], step2 = params[1], eps = params[2], div = params[3], stag = params[4];
    int maxiter = iparams[0], diis_on = iparams[1], nd = iparams[2], projtype = iparams[3];
    int stag_after = iparams[4], check_div = iparams[5], check_stag = iparams[6];
    int solver = iparams[7];
    double *d1 = calloc((size_t)ne, sizeof(double));
    double *d2 = calloc((size_t)ne * ne, sizeof(double));
    diis_t h = {0};
    if (diis_on) {
        h.nd = nd; h.ne = ne; h.np = (size_t)ne * (ne + 1) / 2;
        h.sd1 = calloc((size_t)nd * ne, sizeof(double));
        h.st1 = calloc((size_t)nd * ne, sizeof(double));
        h.sd2 = calloc((size_t)nd * h.np, sizeof(double));
        h.st2 = calloc((size_t)nd * h.np, sizeof(double));
        h.B = calloc((size_t)(nd + 1) * (nd + 1), sizeof(double));
    }
    int iteration = 0, successful = 1, status = 0;
    double current = 0, acc[2];
    for (;;) {
        ++iteration;
        orc_singles(N, o, F, R, t1, t2, d1);
        orc_doubles(N, o, F, R, t1, t2, d2);
        orc_step(N, o, F, t1, t2, d1, d2, step1, step2, projtype, acc);
        double amax = fmax(acc[0], acc[1]);
        if (!(amax < eps) && diis_on) {
            diis_push(&h, N, o, t1, t2, d1, d2, projtype);
            diis_new(&h, N, o, iteration > nd ? nd : iteration, t1, t2, solver);
        }
        orc_energy(N, o, F, R, t1, t2, eref, energy);
        if (trace && iteration <= trace_cap) {
            trace[3 * (iteration - 1) + 0] = acc[0];
            trace[3 * (iteration - 1) + 1] = acc[1];
            trace[3 * (iteration - 1) + 2] = energy[0];
        }
        double previous = current;
        current = amax;
        if (current < previous) ++successful;
        if (current < eps) { status = 1; break; }
        if (check_div && current > div) { status = -2; break; }
        if (iteration + 1 > maxiter) { status = -1; break; }
        if (check_stag && iteration > stag_after &&
            100.0 * successful / iteration <= stag) { status = -3; break; }
    }
    *iterations = iteration;
    free(d1); free(d2);
    if (diis_on) { free(h.sd1); free(h.st1); free(h.sd2); free(h.st2); free(h.B); }
    return status;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
