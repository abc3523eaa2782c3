/*
 * ORACLE — test infrastructure only.  CPU restatement of the reference Gaussium's
 * two-electron repulsion integral path.  tests/ and __graft_entry__.smoke() compare the
 * GPU results with it; the cpu_baseline leg and reference arm of bench.py time it on the
 * host cores.  Nothing in the product library links, loads or calls this file.
 *
 * What it restates (file:line within the reference project):
 *   boys_function            integrals/boys_function.py:4-54   -> oracle_boys_reference
 *   boys_function_recursion  integrals/boys_function.py:57-76  -> boys_down
 *   ObaraSaika.integrate     integrals/twoelectronrepulsion/obara_saika_scheme.py:17-82
 *   ObaraSaika.os_begin      obara_saika_scheme.py:84-115
 *   ObaraSaika.os_recursive  obara_saika_scheme.py:117-146
 *   ObaraSaika.os_int        obara_saika_scheme.py:148-152
 *   os_gaussian_factory      obara_saika_scheme.py:154-195
 *   gaussian_product_coordinate / coordinate_distance  common/vector_manipulation.py:116-120, 21-22
 *
 * The recursion keeps the reference's dispatch order, argument permutations and
 * floating-point operation order, so for identical libm results it reproduces the
 * reference bit for bit (compile with -ffp-contract=off).  The optional memoisation
 * caches os_begin nodes by (m, argument permutation, angular exponents of each original
 * primitive): a node's value is a pure function of that key, so memoised results are
 * bit-identical to the unmemoised recursion, which is the reference's own cost model.
 *
 * boys_mode 0 uses the reference's series (term < 1e-10 stop) for F_L; boys_mode 1 swaps
 * it for an accurate F_L (long-double series, closed form above x = 100); both then run
 * the reference's downward recursion.  Parity is pinned against golden vectors produced
 * by running the reference itself (tests/golden/make_golden.py).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAXM 32

/* ------------------------------------------------------------------ Boys */
double oracle_boys_reference(int v, double x)
{
    /* boys_function.py:28-54 */
    if (x <= 25) {
        int i = 0;
        double ans = 0;
        double g_v = tgamma(v + 0.5);
        for (;;) {
            double seq = (g_v / tgamma(v + i + 1.5)) * pow(x, (double)i);
            if (seq < 1e-10) break;
            ans += seq;
            i += 1;
        }
        ans *= (1.0 / 2) * exp(-x);
        return ans;
    } else {
        int i = 0;
        double ans = 0;
        double g_v = tgamma(v + 0.5);
        for (;;) {
            double seq = (g_v / tgamma(v - i + 1.5)) * pow(x, (double)(-i));
            if (seq < 1e-10) break;
            ans += seq;
            i += 1;
        }
        ans *= (1.0 / 2) * exp(-x);
        ans = (g_v / (2 * pow(x, v + 0.5))) - ans;
        return ans;
    }
}

double oracle_boys_exact(int v, double x)
{
    /* F_v(x) = exp(-x) * sum_i (2x)^i / ((2v+1)(2v+3)...(2v+2i+1)), all terms positive.
     * Above x = 100 the closed form (2v-1)!! sqrt(pi) / (2^(v+1) x^(v+1/2)) is exact to
     * a relative exp(-100). */
    if (x > 100.0) {
        long double df = 1.0L;
        for (int k = 2 * v - 1; k > 1; k -= 2) df *= k;
        long double r = df * sqrtl(3.14159265358979323846264338327950288L) /
                        (powl(2.0L, v + 1) * powl((long double)x, v + 0.5L));
        return (double)r;
    }
    long double term = 1.0L / (2 * v + 1), sum = term, tx = 2.0L * x;
    for (int i = 1; i < 100000; ++i) {
        term *= tx / (2 * v + 2 * i + 1);
        sum += term;
        if (term < sum * 1e-22L) break;
    }
    return (double)(expl(-(long double)x) * sum);
}

static double boys_down(int v, double x, double f_v)
{
    /* boys_function.py:76 */
    return (exp(-x) + 2 * x * f_v) / (2 * v - 1);
}

/* ------------------------------------------------------------------ Obara-Saika port */
typedef struct {
    double a;       /* exponent */
    double r[3];    /* coordinates (bohr) */
    int l[3];       /* integral exponents */
    int orig;       /* which of the four original primitives this one descends from */
} prim_t;

typedef struct {
    double a7;               /* self.a_7 */
    double r7[3];            /* self.r_7 */
    double end[ORACLE_MAXM]; /* self.end_dict */
    int memo;
    int start[4][3];         /* original exponents, bounds of the memo key */
    int span[4];
    int perm_stride, m_stride, size;
    double *val;
    unsigned char *have;
} os_state;

static void gpc(double a, const double *r1, double b, const double *r2, double *out)
{
    /* gaussian_product_coordinate, vector_manipulation.py:116-120 */
    out[0] = (a * r1[0] + b * r2[0]) / (a + b);
    out[1] = (a * r1[1] + b * r2[1]) / (a + b);
    out[2] = (a * r1[2] + b * r2[2]) / (a + b);
}

static double os_begin(os_state *s, int m, const prim_t *g1, const prim_t *g2,
                       const prim_t *g3, const prim_t *g4);

static int perm_id(const prim_t *g1)
{
    /* Positions only ever hold one of four arrangements of the original primitives:
     * (0,1,2,3), (1,0,3,2), (2,3,0,1), (3,2,1,0) -- identified by the first one. */
    return g1->orig;
}

static int memo_key(const os_state *s, int m, const prim_t *g[4])
{
    int key = 0;
    for (int p = 0; p < 4; ++p) {
        const prim_t *q = g[p];
        int o = q->orig;
        int lx = q->l[0], ly = q->l[1], lz = q->l[2];
        int code = (lx * (s->start[o][1] + 1) + ly) * (s->start[o][2] + 1) + lz;
        key = key * s->span[o] + code;   /* ordered by position, so the permutation is implied */
    }
    /* positions are a fixed permutation of the originals given perm_id, but keying by
     * position order already distinguishes them; add perm for safety of the bound. */
    return (m * 4 + perm_id(g[0])) * s->perm_stride + key;
}

static void factory(int r, const prim_t *g1, const prim_t *g2, const prim_t *g3,
                    const prim_t *g4, prim_t out[8])
{
    /* os_gaussian_factory, obara_saika_scheme.py:154-195 */
    out[0] = *g1; out[0].l[r] -= 1;     /* g1x1 */
    out[1] = *g2;
    out[2] = *g3;
    out[3] = *g4;
    out[4] = *g1; out[4].l[r] -= 2;     /* g1x2 */
    out[5] = *g2; out[5].l[r] -= 1;     /* g2x1 */
    out[6] = *g3; out[6].l[r] -= 1;     /* g3x1 */
    out[7] = *g4; out[7].l[r] -= 1;     /* g4x1 */
}

static int os_int(int i) { return i == 0 ? 1 : i; }

static double os_recursive(os_state *s, int r, int m, const prim_t g[8])
{
    /* obara_saika_scheme.py:117-146 */
    double out1 = 0, out2 = 0, out3 = 0, out4 = 0, out5 = 0, out6 = 0, out7 = 0, out8 = 0;
    const prim_t *g1 = &g[0], *g2 = &g[1], *g3 = &g[2], *g4 = &g[3];
    const prim_t *g5 = &g[4], *g6 = &g[5], *g7 = &g[6], *g8 = &g[7];
    double a_1 = g1->a, a_2 = g2->a, a_3 = g3->a, a_4 = g4->a;
    double a_5 = a_1 + a_2;
    double a_6 = a_3 + a_4;
    double r_5[3];
    gpc(a_1, g1->r, a_2, g2->r, r_5);

    if (r_5[r] != g1->r[r])
        out1 = (r_5[r] - g1->r[r]) * os_begin(s, m, g1, g2, g3, g4);
    if (s->r7[r] != r_5[r])
        out2 = (s->r7[r] - r_5[r]) * os_begin(s, m + 1, g1, g2, g3, g4);
    if (g5->l[r] >= 0) {
        out3 = os_int(g1->l[r]) * (1 / (2 * a_5)) * os_begin(s, m, g5, g2, g3, g4);
        out4 = os_int(g1->l[r]) * (s->a7 / (2 * pow(a_5, 2))) * os_begin(s, m + 1, g5, g2, g3, g4);
    }
    if (g6->l[r] >= 0) {
        out5 = os_int(g2->l[r]) * (1 / (2 * a_5)) * os_begin(s, m, g1, g6, g3, g4);
        out6 = os_int(g2->l[r]) * (s->a7 / (2 * pow(a_5, 2))) * os_begin(s, m + 1, g1, g6, g3, g4);
    }
    if (g7->l[r] >= 0)
        out7 = os_int(g3->l[r]) * (1 / (2 * (a_5 + a_6))) * os_begin(s, m + 1, g1, g2, g7, g4);
    if (g8->l[r] >= 0)
        out8 = os_int(g4->l[r]) * (1 / (2 * (a_5 + a_6))) * os_begin(s, m + 1, g1, g2, g3, g8);
    return out1 + out2 + out3 - out4 + out5 - out6 + out7 + out8;
}

static double os_dispatch(os_state *s, int m, const prim_t *g1, const prim_t *g2,
                          const prim_t *g3, const prim_t *g4)
{
    /* obara_saika_scheme.py:84-115 */
    prim_t f[8];
    for (int r = 0; r < 3; ++r)
        if (g1->l[r] > 0) { factory(r, g1, g2, g3, g4, f); return os_recursive(s, r, m, f); }
    for (int r = 0; r < 3; ++r)
        if (g2->l[r] > 0) { factory(r, g2, g1, g4, g3, f); return os_recursive(s, r, m, f); }
    for (int r = 0; r < 3; ++r)
        if (g3->l[r] > 0) { factory(r, g3, g4, g1, g2, f); return os_recursive(s, r, m, f); }
    for (int r = 0; r < 3; ++r)
        if (g4->l[r] > 0) { factory(r, g4, g3, g2, g1, f); return os_recursive(s, r, m, f); }
    return s->end[m];
}

static double os_begin(os_state *s, int m, const prim_t *g1, const prim_t *g2,
                       const prim_t *g3, const prim_t *g4)
{
    if (!s->memo) return os_dispatch(s, m, g1, g2, g3, g4);
    const prim_t *g[4] = {g1, g2, g3, g4};
    int k = memo_key(s, m, g);
    if (s->have[k]) return s->val[k];
    double v = os_dispatch(s, m, g1, g2, g3, g4);
    s->have[k] = 1;
    s->val[k] = v;
    return v;
}

/* ------------------------------------------------------------------ function quartets */
typedef struct {
    const double *centre;  /* nfunc x 3 */
    const int *lmn;        /* nfunc x 3 */
    const double *cnorm;   /* nfunc: Basis.normalisation */
    const int *pstart;     /* nfunc + 1 */
    const double *coef, *expo, *pnorm;  /* primitives: contraction, exponent, normalisation */
} func_table;

static double coordinate_distance(const double *r1, const double *r2)
{
    return sqrt(pow(r1[0] - r2[0], 2) + pow(r1[1] - r2[1], 2) + pow(r1[2] - r2[2], 2));
}

static double integrate(const func_table *t, const int q[4], int boys_mode, int memo,
                        double *scratch_val, unsigned char *scratch_have)
{
    /* ObaraSaika.integrate, obara_saika_scheme.py:17-82 */
    int f[4] = {q[0], q[1], q[2], q[3]};
    int l_total = 0;
    for (int i = 0; i < 4; ++i)
        l_total += t->lmn[3 * f[i]] + t->lmn[3 * f[i] + 1] + t->lmn[3 * f[i] + 2];
    const double *r[4];
    for (int i = 0; i < 4; ++i) r[i] = t->centre + 3 * f[i];
    double n = t->cnorm[f[0]] * t->cnorm[f[1]] * t->cnorm[f[2]] * t->cnorm[f[3]];

    os_state s;
    memset(&s, 0, sizeof(s));
    s.memo = memo;
    if (memo) {
        int stride = 1;
        for (int i = 0; i < 4; ++i) {
            for (int d = 0; d < 3; ++d) s.start[i][d] = t->lmn[3 * f[i] + d];
            s.span[i] = (s.start[i][0] + 1) * (s.start[i][1] + 1) * (s.start[i][2] + 1);
            stride *= s.span[i];
        }
        s.perm_stride = stride;
        s.size = (l_total + 2) * 4 * stride;
        s.val = scratch_val;
        s.have = scratch_have;
    }

    double pi = 3.141592653589793;
    double ans = 0.0;
    for (int i1 = t->pstart[f[0]]; i1 < t->pstart[f[0] + 1]; ++i1)
    for (int i2 = t->pstart[f[1]]; i2 < t->pstart[f[1] + 1]; ++i2)
    for (int i3 = t->pstart[f[2]]; i3 < t->pstart[f[2] + 1]; ++i3)
    for (int i4 = t->pstart[f[3]]; i4 < t->pstart[f[3] + 1]; ++i4) {
        double c_1 = t->coef[i1], c_2 = t->coef[i2], c_3 = t->coef[i3], c_4 = t->coef[i4];
        double n_1 = t->pnorm[i1], n_2 = t->pnorm[i2], n_3 = t->pnorm[i3], n_4 = t->pnorm[i4];
        double contraction = c_1 * c_2 * c_3 * c_4 * n_1 * n_2 * n_3 * n_4 * n;
        double a_1 = t->expo[i1], a_2 = t->expo[i2], a_3 = t->expo[i3], a_4 = t->expo[i4];
        double a_5 = a_1 + a_2;
        double a_6 = a_3 + a_4;
        s.a7 = (a_5 * a_6) / (a_5 + a_6);
        double r_5[3], r_6[3];
        gpc(a_1, r[0], a_2, r[1], r_5);
        gpc(a_3, r[2], a_4, r[3], r_6);
        gpc(a_5, r_5, a_6, r_6, s.r7);
        double r_12 = coordinate_distance(r[0], r[1]);
        double r_34 = coordinate_distance(r[2], r[3]);
        double r_56 = coordinate_distance(r_5, r_6);
        double boys_x = (a_5 * a_6 * pow(r_56, 2)) / (a_5 + a_6);
        double boys_out1 = (2 * pow(pi, 5.0 / 2)) / (a_5 * a_6 * sqrt(a_5 + a_6));
        double boys_out2 = exp(((-a_1 * a_2 * pow(r_12, 2)) / a_5) - ((a_3 * a_4 * pow(r_34, 2)) / a_6));
        double boys_out3 = boys_mode == 0 ? oracle_boys_reference(l_total, boys_x)
                                          : oracle_boys_exact(l_total, boys_x);
        s.end[l_total] = boys_out1 * boys_out2 * boys_out3;
        for (int m = l_total; m >= 1;) {
            boys_out3 = boys_down(m, boys_x, boys_out3);
            m -= 1;
            s.end[m] = boys_out1 * boys_out2 * boys_out3;
        }
        prim_t g[4];
        const int idx[4] = {i1, i2, i3, i4};
        for (int i = 0; i < 4; ++i) {
            g[i].a = t->expo[idx[i]];
            for (int d = 0; d < 3; ++d) { g[i].r[d] = r[i][d]; g[i].l[d] = t->lmn[3 * f[i] + d]; }
            g[i].orig = i;
        }
        if (memo) memset(s.have, 0, (size_t)s.size);
        ans += contraction * os_begin(&s, 0, &g[0], &g[1], &g[2], &g[3]);
    }
    return ans;
}

typedef struct {
    const func_table *t;
    const int *quartets;
    long begin, end;
    int boys_mode, memo;
    double *out;
    long *next;     /* shared work counter: quartets are handed out 8 at a time */
} job_t;

#define MEMO_CAP (1 << 20)

static void *worker(void *arg)
{
    job_t *j = (job_t *)arg;
    double *val = NULL;
    unsigned char *have = NULL;
    if (j->memo) {
        val = (double *)malloc(sizeof(double) * MEMO_CAP);
        have = (unsigned char *)malloc(MEMO_CAP);
    }
    for (;;) {
        long i0 = __sync_fetch_and_add(j->next, 8);
        if (i0 >= j->end) break;
        long i1 = i0 + 8 < j->end ? i0 + 8 : j->end;
        for (long i = i0; i < i1; ++i)
            j->out[i] = integrate(j->t, j->quartets + 4 * i, j->boys_mode, j->memo, val, have);
    }
    free(val);
    free(have);
    return NULL;
}

/* Evaluate nq function quartets.  Returns 0, or -1 on bad arguments (L too large for
 * the memo capacity or the Boys table). */
int oracle_eri_functions(int nfunc, const double *centre, const int *lmn, const double *cnorm,
                         const int *pstart, const double *coef, const double *expo,
                         const double *pnorm, long nq, const int *quartets, int boys_mode,
                         int memo, int nthreads, double *out)
{
    func_table t = {centre, lmn, cnorm, pstart, coef, expo, pnorm};
    for (long i = 0; i < nq; ++i) {
        int lt = 0;
        long span = 1;
        for (int k = 0; k < 4; ++k) {
            int fi = quartets[4 * i + k];
            if (fi < 0 || fi >= nfunc) return -1;
            lt += lmn[3 * fi] + lmn[3 * fi + 1] + lmn[3 * fi + 2];
            span *= (long)(lmn[3 * fi] + 1) * (lmn[3 * fi + 1] + 1) * (lmn[3 * fi + 2] + 1);
        }
        if (lt + 2 > ORACLE_MAXM) return -1;
        if (memo && (long)(lt + 2) * 4 * span > MEMO_CAP) return -1;
    }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (nq < nthreads) nthreads = nq > 0 ? (int)nq : 1;
    pthread_t th[256];
    job_t jobs[256];
    long next = 0;
    for (int k = 0; k < nthreads; ++k) {
        jobs[k].t = &t;
        jobs[k].quartets = quartets;
        jobs[k].begin = 0;
        jobs[k].end = nq;
        jobs[k].boys_mode = boys_mode;
        jobs[k].memo = memo;
        jobs[k].out = out;
        jobs[k].next = &next;
    }
    if (nthreads == 1) {
        worker(&jobs[0]);
        return 0;
    }
    for (int k = 0; k < nthreads; ++k) pthread_create(&th[k], NULL, worker, &jobs[k]);
    for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
    return 0;
}
