/*
 * wilson_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference Wilson-fermion operator and CG solver
 * (CHN-ChenYi/IPCC2021-Final).  It is the oracle the CUDA library is tested
 * against: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark load it.  Nothing in the product links against it.
 *
 * Parity pinning: this restatement is checked against golden vectors written
 * by the reference's own sources (compiled single-rank), stored under
 * tests/golden/.
 *
 * Layout (reference, include/operator.h:56-67, src/lattice_fermion.cpp:15-22,
 * src/load_gauge.cpp:141-161):
 *   site (x,y,z,t), x fastest; lex = x + Lx*(y + Ly*(z + Lz*t));
 *   eo  = lex/2 + ((x+y+z+t)&1) * V/2       (requires Lx even)
 *   fermion: psi[(eo*12 + spin*3 + colour)]  complex double (re,im pairs)
 *   gauge:   U[mu][(eo*9 + row*3 + col)]     = U_mu(x), link x -> x+mu
 * Boundary conditions: periodic in all four directions.
 *
 * Operator (src/dslash.cpp:38-1249 scalar form, src/invert.cpp:138-156):
 *   M psi = (4+m) psi - 1/2 sum_mu [ (1 - g_mu) U_mu(x) psi(x+mu)
 *                                  + (1 + g_mu) U_mu(x-mu)^dag psi(x-mu) ]
 *   M^dag flips the sign of every g_mu (flag = -1, dslash.cpp:92).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cplx;

static inline cplx c_add(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cplx c_sub(cplx a, cplx b) { cplx r = {a.re - b.re, a.im - b.im}; return r; }
static inline cplx c_mul(cplx a, cplx b)
{
    cplx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
    return r;
}
static inline cplx c_conjmul(cplx a, cplx b) /* conj(a) * b */
{
    cplx r = {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
    return r;
}
static inline cplx c_scale(cplx a, double s) { cplx r = {a.re * s, a.im * s}; return r; }
static inline cplx c_i(cplx a) { cplx r = {-a.im, a.re}; return r; } /* i*a */

int wo_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* site2eoindex of include/operator.h:62-67 for a single rank. */
static inline long eo_index(const int *L, int x, int y, int z, int t)
{
    long lex = x + (long)L[0] * (y + (long)L[1] * (z + (long)L[2] * t));
    long vh = (long)L[0] * L[1] * L[2] * L[3] / 2;
    return lex / 2 + ((x + y + z + t) & 1) * vh;
}

/*
 * Hopping term for one output site (gather form).  The per-direction
 * projectors and reconstructions follow src/dslash.cpp:544-873 exactly:
 * the half-spinor h = P psi(neighbour) is multiplied by W (U_mu(x) forward,
 * U_mu(x-mu)^dag backward), and t = W h feeds the four spin components.
 * The -1/2 is applied once at the end (the reference applies it per term).
 * src holds sites from eo index src_off on (0: a full-lattice array; Vh: an
 * array of the odd sites only).
 */
static void hop_site(const cplx *src, long src_off, const cplx *const U[4], const int *L, double flag,
                     int x, int y, int z, int t, cplx out[12])
{
    int c[4] = {x, y, z, t};
    cplx acc[12];
    memset(acc, 0, sizeof(acc));
    long here = eo_index(L, x, y, z, t);
    for (int mu = 0; mu < 4; ++mu) {
        for (int dir = 0; dir < 2; ++dir) { /* 0 forward, 1 backward */
            int n[4] = {c[0], c[1], c[2], c[3]};
            n[mu] = dir == 0 ? (c[mu] + 1) % L[mu] : (c[mu] - 1 + L[mu]) % L[mu];
            long nb = eo_index(L, n[0], n[1], n[2], n[3]);
            const cplx *s = src + (nb - src_off) * 12;
            /* link: forward U_mu(x) at this site; backward U_mu(x-mu) at nb */
            const cplx *W = U[mu] + (dir == 0 ? here : nb) * 9;
            /* sign of the gamma term: (1 - g) forward, (1 + g) backward, times flag */
            double sg = (dir == 0 ? -1.0 : 1.0) * flag;
            cplx h0[3], h1[3];
            for (int k = 0; k < 3; ++k) {
                cplx s0 = s[0 * 3 + k], s1 = s[1 * 3 + k], s2 = s[2 * 3 + k], s3 = s[3 * 3 + k];
                switch (mu) {
                case 0: /* x: h0 = s0 + sg*i*s3, h1 = s1 + sg*i*s2 */
                    h0[k] = c_add(s0, c_scale(c_i(s3), sg));
                    h1[k] = c_add(s1, c_scale(c_i(s2), sg));
                    break;
                case 1: /* y: h0 = s0 - sg*s3, h1 = s1 + sg*s2 */
                    h0[k] = c_sub(s0, c_scale(s3, sg));
                    h1[k] = c_add(s1, c_scale(s2, sg));
                    break;
                case 2: /* z: h0 = s0 + sg*i*s2, h1 = s1 - sg*i*s3 */
                    h0[k] = c_add(s0, c_scale(c_i(s2), sg));
                    h1[k] = c_sub(s1, c_scale(c_i(s3), sg));
                    break;
                default: /* t: h0 = s0 + sg*s2, h1 = s1 + sg*s3 */
                    h0[k] = c_add(s0, c_scale(s2, sg));
                    h1[k] = c_add(s1, c_scale(s3, sg));
                    break;
                }
            }
            cplx t0[3], t1[3];
            for (int a = 0; a < 3; ++a) {
                cplx r0 = {0, 0}, r1 = {0, 0};
                for (int b = 0; b < 3; ++b) {
                    if (dir == 0) {
                        r0 = c_add(r0, c_mul(W[a * 3 + b], h0[b]));
                        r1 = c_add(r1, c_mul(W[a * 3 + b], h1[b]));
                    } else {
                        r0 = c_add(r0, c_conjmul(W[b * 3 + a], h0[b]));
                        r1 = c_add(r1, c_conjmul(W[b * 3 + a], h1[b]));
                    }
                }
                t0[a] = r0;
                t1[a] = r1;
            }
            /* lower spin components: -sg folds in (1 - g) vs (1 + g) and flag */
            double lg = -sg;
            for (int a = 0; a < 3; ++a) {
                acc[0 * 3 + a] = c_add(acc[0 * 3 + a], t0[a]);
                acc[1 * 3 + a] = c_add(acc[1 * 3 + a], t1[a]);
                switch (mu) {
                case 0: /* x fwd: d2 += i t1, d3 += i t0 (flag=+1) */
                    acc[2 * 3 + a] = c_add(acc[2 * 3 + a], c_scale(c_i(t1[a]), lg));
                    acc[3 * 3 + a] = c_add(acc[3 * 3 + a], c_scale(c_i(t0[a]), lg));
                    break;
                case 1: /* y fwd: d2 -= t1, d3 += t0 */
                    acc[2 * 3 + a] = c_sub(acc[2 * 3 + a], c_scale(t1[a], lg));
                    acc[3 * 3 + a] = c_add(acc[3 * 3 + a], c_scale(t0[a], lg));
                    break;
                case 2: /* z fwd: d2 += i t0, d3 -= i t1 */
                    acc[2 * 3 + a] = c_add(acc[2 * 3 + a], c_scale(c_i(t0[a]), lg));
                    acc[3 * 3 + a] = c_sub(acc[3 * 3 + a], c_scale(c_i(t1[a]), lg));
                    break;
                default: /* t fwd: d2 -= t0, d3 -= t1 */
                    acc[2 * 3 + a] = c_sub(acc[2 * 3 + a], c_scale(t0[a], lg));
                    acc[3 * 3 + a] = c_sub(acc[3 * 3 + a], c_scale(t1[a], lg));
                    break;
                }
            }
        }
    }
    for (int k = 0; k < 12; ++k)
        out[k] = c_scale(acc[k], -0.5);
}

/*
 * DslashoffdNew (src/dslash_new.cpp:1341-2677) / Dslashoffd (src/dslash.cpp:38-1249):
 * dest is zeroed over the whole lattice, then the parity-cb half receives the
 * hopping term of the parity-(1-cb) half of src.
 */
void wo_dslash_offd(const double *src_d, double *dest_d, const double *const gauge_d[4],
                    const int *L, int dag, int cb)
{
    const cplx *src = (const cplx *)src_d;
    cplx *dest = (cplx *)dest_d;
    const cplx *U[4] = {(const cplx *)gauge_d[0], (const cplx *)gauge_d[1],
                        (const cplx *)gauge_d[2], (const cplx *)gauge_d[3]};
    long V = (long)L[0] * L[1] * L[2] * L[3];
    double flag = dag ? -1.0 : 1.0;
    memset(dest, 0, sizeof(cplx) * 12 * V);
    long rows = (long)L[1] * L[2] * L[3];
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        int y = (int)(r % L[1]);
        int z = (int)((r / L[1]) % L[2]);
        int t = (int)(r / ((long)L[1] * L[2]));
        for (int x = 0; x < L[0]; ++x) {
            if (((x + y + z + t) & 1) != cb)
                continue;
            hop_site(src, 0, U, L, flag, x, y, z, t, dest + eo_index(L, x, y, z, t) * 12);
        }
    }
}

/* DslashEEOONew (src/dslash_new.cpp:1301-1338): dest = (4+m) src on all sites. */
void wo_dslash_eeoo(const double *src, double *dest, const int *L, double mass)
{
    long n = (long)L[0] * L[1] * L[2] * L[3] * 24;
    double a = 4.0 + mass;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i)
        dest[i] = a * src[i];
}

/*
 * DslashNew (src/invert.cpp:138-156): full M (dag=0) or M^dag (dag=1),
 * fused per site: dest = (4+m) src + hop(src) over both parities.
 */
void wo_dslash_full(const double *src_d, double *dest_d, const double *const gauge_d[4],
                    const int *L, double mass, int dag)
{
    const cplx *src = (const cplx *)src_d;
    cplx *dest = (cplx *)dest_d;
    const cplx *U[4] = {(const cplx *)gauge_d[0], (const cplx *)gauge_d[1],
                        (const cplx *)gauge_d[2], (const cplx *)gauge_d[3]};
    double flag = dag ? -1.0 : 1.0;
    double a = 4.0 + mass;
    long rows = (long)L[1] * L[2] * L[3];
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        int y = (int)(r % L[1]);
        int z = (int)((r / L[1]) % L[2]);
        int t = (int)(r / ((long)L[1] * L[2]));
        for (int x = 0; x < L[0]; ++x) {
            long e = eo_index(L, x, y, z, t);
            cplx h[12];
            hop_site(src, 0, U, L, flag, x, y, z, t, h);
            for (int k = 0; k < 12; ++k)
                dest[e * 12 + k] = c_add(c_scale(src[e * 12 + k], a), h[k]);
        }
    }
}

/* norm_2 (include/operator_mpi.h:15-46): sum |a_i|^2 over n complex entries. */
double wo_norm2(const double *a, long n)
{
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < 2 * n; ++i)
        s += a[i] * a[i];
    return s;
}

/* vector_p (include/operator_mpi.h:48-79): sum conj(a_i) b_i; result in out[2]. */
void wo_dot(const double *a, const double *b, long n, double *out)
{
    double re = 0.0, im = 0.0;
#pragma omp parallel for reduction(+ : re, im) schedule(static)
    for (long i = 0; i < n; ++i) {
        re += a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1];
        im += a[2 * i] * b[2 * i + 1] - a[2 * i + 1] * b[2 * i];
    }
    out[0] = re;
    out[1] = im;
}

/* n values rand()/RAND_MAX from the current rand() stream: the source of
 * src/main.cpp:82-85 (re, im interleaved) after srand(rank + seed). */
void wo_rand_fill(double *out, long n)
{
    for (long i = 0; i < n; ++i)
        out[i] = (double)rand() / RAND_MAX;
}

/* Fill the CG initial guess as src/invert.cpp:42-44 does: real part rand()/RAND_MAX. */
void wo_srand(unsigned seed) { srand(seed); }
void wo_rand_guess(double *x, long n)
{
    for (long i = 0; i < n; ++i) {
        x[2 * i] = 1.0 * rand() / RAND_MAX;
        x[2 * i + 1] = 0.0;
    }
}

/*
 * CGinvert (src/invert.cpp:25-121): CG on the normal equations
 * M^dag M x = M^dag b over the full lattice, complex alpha/beta, stopping when
 * the absolute normal residual |r| < accuracy.  `dest` holds the initial guess
 * on entry (the reference overwrites it with rand() values first; callers that
 * want that call wo_rand_guess).  Returns the iteration count f at which it
 * stopped (max-1 when it did not converge); *rsd_out = final |r|.
 */
int wo_cg_ref(const double *src, double *dest, const double *const gauge[4], const int *L,
              double mass, int max, double accuracy, double *rsd_out)
{
    long V = (long)L[0] * L[1] * L[2] * L[3];
    long n = V * 12;
    size_t bytes = sizeof(double) * 2 * (size_t)n;
    double *r0 = (double *)malloc(bytes), *q = (double *)malloc(bytes);
    double *qq = (double *)malloc(bytes), *p = (double *)malloc(bytes);
    double *Mdb = (double *)malloc(bytes), *tmp = (double *)malloc(bytes);
    double r1[2] = {0, 0}, rsd = 0.0;
    int f, iters = 0;

    wo_dslash_full(src, Mdb, gauge, L, mass, 1);
    wo_dslash_full(dest, tmp, gauge, L, mass, 0);
    wo_dslash_full(tmp, r0, gauge, L, mass, 1);
    for (long i = 0; i < 2 * n; ++i)
        r0[i] = Mdb[i] - r0[i];

    for (f = 1; f < max; ++f) {
        if (f == 1) {
            memcpy(p, r0, bytes);
        } else {
            double rr[2];
            wo_dot(r0, r0, n, rr);
            /* beta = (r,r)/r1, complex division */
            double den = r1[0] * r1[0] + r1[1] * r1[1];
            double br = (rr[0] * r1[0] + rr[1] * r1[1]) / den;
            double bi = (rr[1] * r1[0] - rr[0] * r1[1]) / den;
#pragma omp parallel for schedule(static)
            for (long i = 0; i < n; ++i) {
                double pr = p[2 * i], pi = p[2 * i + 1];
                p[2 * i] = r0[2 * i] + br * pr - bi * pi;
                p[2 * i + 1] = r0[2 * i + 1] + br * pi + bi * pr;
            }
        }
        wo_dslash_full(p, qq, gauge, L, mass, 0);
        wo_dslash_full(qq, q, gauge, L, mass, 1);
        wo_dot(r0, r0, n, r1);
        double pq[2];
        wo_dot(p, q, n, pq);
        double den = pq[0] * pq[0] + pq[1] * pq[1];
        double ar = (r1[0] * pq[0] + r1[1] * pq[1]) / den;
        double ai = (r1[1] * pq[0] - r1[0] * pq[1]) / den;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
            double pr = p[2 * i], pi = p[2 * i + 1];
            double qr = q[2 * i], qi = q[2 * i + 1];
            dest[2 * i] += ar * pr - ai * pi;
            dest[2 * i + 1] += ar * pi + ai * pr;
            r0[2 * i] -= ar * qr - ai * qi;
            r0[2 * i + 1] -= ar * qi + ai * qr;
        }
        rsd = sqrt(wo_norm2(r0, n));
        iters = f;
        if (rsd < accuracy)
            break;
    }
    free(r0); free(q); free(qq); free(p); free(Mdb); free(tmp);
    if (rsd_out)
        *rsd_out = rsd;
    return iters;
}

/*
 * One parity of the hopping term on half-lattice arrays: out[i] (the site of
 * parity cb with eo index cb*Vh + i) = -1/2 sum_mu hop(in), where in[j] is the
 * site of parity 1-cb with eo index (1-cb)*Vh + j.  This is the interior of
 * DslashoffdNew (src/dslash_new.cpp:1341-2677) without its memset of the
 * other parity.  flag -1 gives the hopping term of M^dag.
 */
static void hop_half(const cplx *in, cplx *out, const cplx *const U[4], const int *L, double flag, int cb)
{
    long vh = (long)L[0] * L[1] * L[2] * L[3] / 2;
    long rows = (long)L[1] * L[2] * L[3];
#pragma omp parallel for schedule(static)
    for (long r = 0; r < rows; ++r) {
        int y = (int)(r % L[1]);
        int z = (int)((r / L[1]) % L[2]);
        int t = (int)(r / ((long)L[1] * L[2]));
        for (int x = 0; x < L[0]; ++x) {
            if (((x + y + z + t) & 1) != cb)
                continue;
            hop_site(in, (1 - cb) * vh, U, L, flag, x, y, z, t, out + (eo_index(L, x, y, z, t) - cb * vh) * 12);
        }
    }
}

/*
 * Schur complement on the even sites: out = a*in - H_eo H_oe in / a, with
 * H = -1/2 D the hopping term (M = a + H, a = 4 + m).  flag -1 gives the
 * adjoint, a - (H^dag)_eo (H^dag)_oe / a.  tmp: Vh*12 entries.
 */
static void schur_apply(const cplx *in, cplx *out, cplx *tmp, const cplx *const U[4], const int *L, double a,
                        double flag)
{
    long n = (long)L[0] * L[1] * L[2] * L[3] / 2 * 12;
    hop_half(in, tmp, U, L, flag, 1);
    hop_half(tmp, out, U, L, flag, 0);
    double ia = 1.0 / a;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        out[i].re = a * in[i].re - ia * out[i].re;
        out[i].im = a * in[i].im - ia * out[i].im;
    }
}

/*
 * Even-odd (Schur) preconditioned CG -- the solver form of the IPCC 2021
 * problem statement (doc/IPCC_2021.pdf, p.9-11), used here to produce
 * reference solutions cheaply at large volumes; CGinvert (src/invert.cpp:25-121,
 * wo_cg_ref above) solves the same M x = b on the full lattice.
 *   b^_e = b_e - H_eo b_o / a;  CG on  M^dag M^ x_e = M^dag b^_e  (real alpha,
 *   beta) until |r| <= tol |M^dag b^_e|;  x_o = (b_o - H_oe x_e) / a.
 * dest receives the full-lattice solution (reference layout, even sites
 * first).  *true_res_out = |b - M x| / |b| recomputed with the full operator.
 * Returns the iteration count (max when it did not converge).
 */
int wo_cg_eo(const double *src_d, double *dest_d, const double *const gauge_d[4], const int *L, double mass,
             int max, double tol, double *true_res_out)
{
    const cplx *src = (const cplx *)src_d;
    cplx *dest = (cplx *)dest_d;
    const cplx *U[4] = {(const cplx *)gauge_d[0], (const cplx *)gauge_d[1],
                        (const cplx *)gauge_d[2], (const cplx *)gauge_d[3]};
    long V = (long)L[0] * L[1] * L[2] * L[3], vh = V / 2, n = vh * 12;
    double a = 4.0 + mass;
    size_t bytes = sizeof(cplx) * (size_t)n;
    cplx *bh = (cplx *)malloc(bytes), *r = (cplx *)malloc(bytes), *p = (cplx *)malloc(bytes);
    cplx *q = (cplx *)malloc(bytes), *q2 = (cplx *)malloc(bytes), *tmp = (cplx *)malloc(bytes);
    cplx *x = dest; /* even half of dest */
    const cplx *b_e = src, *b_o = src + n;
    int it = 0;

    hop_half(b_o, tmp, U, L, 1.0, 0);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        bh[i].re = b_e[i].re - tmp[i].re / a;
        bh[i].im = b_e[i].im - tmp[i].im / a;
    }
    schur_apply(bh, r, tmp, U, L, a, -1.0);
    memset(x, 0, bytes);
    memcpy(p, r, bytes);
    double rr = wo_norm2((const double *)r, n);
    const double stop = tol * tol * rr;
    while (it < max && rr > stop) {
        schur_apply(p, q, tmp, U, L, a, 1.0);
        schur_apply(q, q2, tmp, U, L, a, -1.0);
        double alpha = rr / wo_norm2((const double *)q, n);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
            x[i].re += alpha * p[i].re;
            x[i].im += alpha * p[i].im;
            r[i].re -= alpha * q2[i].re;
            r[i].im -= alpha * q2[i].im;
        }
        double rr_new = wo_norm2((const double *)r, n);
        double beta = rr_new / rr;
        rr = rr_new;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; ++i) {
            p[i].re = r[i].re + beta * p[i].re;
            p[i].im = r[i].im + beta * p[i].im;
        }
        ++it;
    }
    /* x_o = (b_o - H_oe x_e) / a */
    hop_half(x, tmp, U, L, 1.0, 1);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        dest[n + i].re = (b_o[i].re - tmp[i].re) / a;
        dest[n + i].im = (b_o[i].im - tmp[i].im) / a;
    }
    if (true_res_out) {
        cplx *full = (cplx *)malloc(2 * bytes);
        wo_dslash_full(dest_d, (double *)full, gauge_d, L, mass, 0);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < 2 * n; ++i) {
            full[i].re = src[i].re - full[i].re;
            full[i].im = src[i].im - full[i].im;
        }
        double nb = wo_norm2(src_d, 2 * n);
        *true_res_out = sqrt(wo_norm2((const double *)full, 2 * n) / (nb > 0 ? nb : 1.0));
        free(full);
    }
    free(bh); free(r); free(p); free(q); free(q2); free(tmp);
    return it;
}

/*
 * check (src/check.cpp:28-110): the residual report of the reference.
 * out[0]=|b| out[1]=|x| out[2..3]=(Mb,Mb) out[4..5]=(b,M^dag M b)
 * out[6..7]=(Mx,Mx) out[8..9]=(x,M^dag M x) out[10]=|Mx-b| out[11]=|M^dag M x - M^dag b|
 */
void wo_check(const double *b, const double *x, const double *const gauge[4], const int *L,
              double mass, double *out)
{
    long V = (long)L[0] * L[1] * L[2] * L[3];
    long n = V * 12;
    size_t bytes = sizeof(double) * 2 * (size_t)n;
    double *Mb = (double *)malloc(bytes), *Mdb = (double *)malloc(bytes);
    double *MMb = (double *)malloc(bytes), *Mx = (double *)malloc(bytes);
    double *MMx = (double *)malloc(bytes), *tmp = (double *)malloc(bytes);
    out[0] = sqrt(wo_norm2(b, n));
    out[1] = sqrt(wo_norm2(x, n));
    wo_dslash_full(b, Mb, gauge, L, mass, 0);
    wo_dslash_full(b, Mdb, gauge, L, mass, 1);
    wo_dslash_full(Mb, MMb, gauge, L, mass, 1);
    wo_dslash_full(x, Mx, gauge, L, mass, 0);
    for (long i = 0; i < 2 * n; ++i)
        tmp[i] = Mx[i] - b[i];
    out[10] = sqrt(wo_norm2(tmp, n));
    wo_dslash_full(Mx, MMx, gauge, L, mass, 1);
    for (long i = 0; i < 2 * n; ++i)
        tmp[i] = MMx[i] - Mdb[i];
    out[11] = sqrt(wo_norm2(tmp, n));
    wo_dot(Mb, Mb, n, out + 2);
    wo_dot(b, MMb, n, out + 4);
    wo_dot(Mx, Mx, n, out + 6);
    wo_dot(x, MMx, n, out + 8);
    free(Mb); free(Mdb); free(MMb); free(Mx); free(MMx); free(tmp);
}
