/* CPU oracle: FP64 restatement of 3DDG's DG right-hand side and RK33 loop.
 *
 * TEST INFRASTRUCTURE ONLY (see dg_oracle.h).  Each routine names the
 * reference code it restates.  Deliberate differences from the reference:
 *   - the per-line linear solve uses Gaussian elimination with partial
 *     pivoting instead of the pivoted Householder QR of cppsrc/Matrix.h:289-445.
 *     Both solve the same non-singular system to rounding; the reference's
 *     rank cutoff (aTol = 1e-6 on row norms, cppsrc/Matrix.h:320) is not
 *     restated, so inputs must keep M*q*w row norms above 1e-6 (millimetre /
 *     microsecond units do; SI units do not for the mass equation);
 *   - element constants (rho0, c0, B/A, D) are per problem, as the reference's
 *     Grid constructor sets them (cppsrc/Grid.cpp:176);
 *   - the tone-burst boundary source does not exist in the reference; it is
 *     restated here from this package's definition (exterior state on one
 *     face, written into that face's halo nodes before each stage).
 */
#include "dg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define DG_PI 3.14159265358979323846

enum { F_RHO = 0, F_U0 = 1, F_Q0 = 4, NF = 7 };

typedef struct {
    double* f; /* [NF][nelh][K3] */
} grid_t;

struct dgo_sim {
    dgo_params p;
    int K, K3, N;
    int E[3], H[3];
    size_t nelh;
    double M[100], S[100], zeros[10];
    double* sigma;  /* per element incl. halo */
    double* coords; /* [3][nelh][K3] */
    grid_t g[4];    /* 0 = myGrid, 1 = myGrid2, 2 = k1, 3 = k2 (cppsrc/driver.cpp:210-213) */
    int cur;        /* grid holding the latest state (the driver's newGrid) */
    double t;
    double* line_tmp;
};

static inline size_t eidx(const dgo_sim* s, int i, int j, int k)
{
    return ((size_t)i * s->H[1] + j) * s->H[2] + k;
}

static inline double* fld(const dgo_sim* s, const grid_t* g, int f, size_t e)
{
    return g->f + ((size_t)f * s->nelh + e) * s->K3;
}

static inline int nidx(int K, const int c[3]) { return (c[0] * K + c[1]) * K + c[2]; }

/* cppsrc/kernelFuncs.cpp:19-20 (scalar) and :13-15 (vector, same op order) */
static inline double momentum(double u, double d, double c, double r0, double ba)
{
    (void)u;
    return (d + d * d * ba * .5 * (1.0 / r0)) * (c * c / r0);
}

/* cppsrc/kernelFuncs.cpp:23-29 */
static inline double mass(double u, double d, double c, double r0, double ba)
{
    (void)c;
    if (ba == 0.0) return u * r0;
    return u * (d + r0);
}

/* Solve A x = b for a KxK system by Gaussian elimination with partial pivoting
   (stands in for Matrix::operator/, cppsrc/Matrix.h:625-628). */
static void solve(int K, const double* Ain, const double* b, double* x)
{
    double A[100], r[10];
    memcpy(A, Ain, sizeof(double) * K * K);
    memcpy(r, b, sizeof(double) * K);
    for (int c = 0; c < K; c++) {
        int piv = c;
        for (int i = c + 1; i < K; i++)
            if (fabs(A[i * K + c]) > fabs(A[piv * K + c])) piv = i;
        if (piv != c) {
            for (int j = 0; j < K; j++) {
                double t = A[c * K + j];
                A[c * K + j] = A[piv * K + j];
                A[piv * K + j] = t;
            }
            double t = r[c];
            r[c] = r[piv];
            r[piv] = t;
        }
        for (int i = c + 1; i < K; i++) {
            double m = A[i * K + c] / A[c * K + c];
            for (int j = c; j < K; j++) A[i * K + j] -= m * A[c * K + j];
            r[i] -= m * r[c];
        }
    }
    for (int i = K - 1; i >= 0; i--) {
        double v = r[i];
        for (int j = i + 1; j < K; j++) v -= A[i * K + j] * x[j];
        x[i] = v / A[i * K + i];
    }
}

/* Block::setZero over every element including the halo ring
   (cppsrc/Block.cpp:297-309). */
static void set_zero(dgo_sim* s, grid_t* g)
{
    memset(g->f, 0, sizeof(double) * NF * s->nelh * s->K3);
}

/* Grid::periodicSelf (cppsrc/Grid.cpp:385-440): periodic halos take the
   opposite interior element's node data; other halos are left untouched. */
static void communicate(dgo_sim* s, grid_t* g)
{
    const int* E = s->E;
    for (int i = 0; i < s->H[0]; i++)
        for (int j = 0; j < s->H[1]; j++)
            for (int k = 0; k < s->H[2]; k++) {
                int fi = i, fj = j, fk = k, send = 0;
                if (i == 0) { fi = E[0]; send = s->p.periodic[0]; }
                else if (i == E[0] + 1) { fi = 1; send = s->p.periodic[0]; }
                else if (j == 0) { fj = E[1]; send = s->p.periodic[1]; }
                else if (j == E[1] + 1) { fj = 1; send = s->p.periodic[1]; }
                else if (k == 0) { fk = E[2]; send = s->p.periodic[2]; }
                else if (k == E[2] + 1) { fk = 1; send = s->p.periodic[2]; }
                if (!send) continue;
                size_t to = eidx(s, i, j, k), from = eidx(s, fi, fj, fk);
                for (int f = 0; f < NF; f++)
                    memcpy(fld(s, g, f, to), fld(s, g, f, from), sizeof(double) * s->K3);
            }
}

static double burst(const dgo_params* p, double t)
{
    double T = p->src_cycles / p->src_freq;
    if (t < 0.0 || t > T) return 0.0;
    double w = sin(DG_PI * t / T);
    return p->src_amp * w * w * sin(2.0 * DG_PI * p->src_freq * t + p->src_phase);
}

/* Tone-burst source: exterior state on face src_face at time t, written into
   the face nodes of that face's halo elements. */
static void apply_source(dgo_sim* s, grid_t* g, double t)
{
    const dgo_params* p = &s->p;
    if (p->src_face < 0) return;
    int ax = p->src_face / 2, side = p->src_face % 2;
    int a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
    int K = s->K, N = s->N;
    double pval = burst(p, t);
    double drho = pval / (p->c0 * p->c0);
    double un = (side == 0 ? 1.0 : -1.0) * pval / (p->rho0 * p->c0);
    double ctr1 = p->corner[a1] + 0.5 * s->E[a1] * p->elem_width[a1];
    double ctr2 = p->corner[a2] + 0.5 * s->E[a2] * p->elem_width[a2];
    int hi = side == 0 ? 0 : s->E[ax] + 1;
    for (int b1 = 1; b1 <= s->E[a1]; b1++)
        for (int b2 = 1; b2 <= s->E[a2]; b2++) {
            int ec[3];
            ec[ax] = hi; ec[a1] = b1; ec[a2] = b2;
            size_t e = eidx(s, ec[0], ec[1], ec[2]);
            for (int n1 = 0; n1 < K; n1++)
                for (int n2 = 0; n2 < K; n2++) {
                    int c[3];
                    c[ax] = side == 0 ? N : 0; c[a1] = n1; c[a2] = n2;
                    int n = nidx(K, c);
                    double ap = 1.0;
                    if (p->src_radius > 0.0) {
                        double x1 = s->coords[((size_t)a1 * s->nelh + e) * s->K3 + n] - ctr1;
                        double x2 = s->coords[((size_t)a2 * s->nelh + e) * s->K3 + n] - ctr2;
                        if (x1 * x1 + x2 * x2 > p->src_radius * p->src_radius) ap = 0.0;
                    }
                    fld(s, g, F_RHO, e)[n] = drho * ap;
                    fld(s, g, F_U0 + ax, e)[n] = un * ap;
                }
        }
}

static size_t ax_stride(const dgo_sim* s, int axis)
{
    if (axis == 0) return (size_t)s->H[1] * s->H[2];
    if (axis == 1) return (size_t)s->H[2];
    return 1;
}

/* Element::OperateUFromV (cppsrc/Element.cpp:475-620) over the interior
   elements of a block (cppsrc/Block.cpp:343-356): upwind impedance flux at
   both faces, volume term S q f, line solve with M q w, accumulate. */
static void op_u_from_v(dgo_sim* s, grid_t* dst, grid_t* src, int axis, int mode, size_t e)
{
    const dgo_params* p = &s->p;
    const int K = s->K, N = s->N;
    const double r0 = p->rho0, c0 = p->c0, ba = p->b_over_a;
    const double w = p->elem_width[axis];
    const size_t st = ax_stride(s, axis);
    const double q = mode == 0 ? r0 : 1.0 / r0;
    double (*kF)(double, double, double, double, double) = mode == 0 ? momentum : mass;
    double (*kF2)(double, double, double, double, double) = mode == 0 ? mass : momentum;
    double A[100], Sq[100];
    for (int i = 0; i < K * K; i++) A[i] = w * (q * s->M[i]);
    for (int i = 0; i < K * K; i++) Sq[i] = q * s->S[i];
    const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
    const double* rs = fld(s, src, F_RHO, e);
    const double* us = fld(s, src, F_U0 + axis, e);
    for (int l1 = 0; l1 < K; l1++)
        for (int l2 = 0; l2 < K; l2++) {
            int c[3], oc[3];
            c[o1] = oc[o1] = l1;
            c[o2] = oc[o2] = l2;
            double flux[10] = {0}, dR[10], vel[10], f[10], rhs[10], res[10];
            /* left face, other = neighbour k-1/j-1/i-1 */
            size_t eo = e - st;
            const double* ro = fld(s, src, F_RHO, eo);
            const double* uo = fld(s, src, F_U0 + axis, eo);
            c[axis] = 0;
            oc[axis] = N;
            double z1 = r0 * c0, z2 = r0 * c0, r1 = r0, r2 = r0;
            double c1, c2, c3, c4;
            if (mode == 0) {
                c1 = z1 * r2 / (z1 + z2); c2 = z2 * r1 / (z1 + z2);
                c3 = z1 * z2 / r2 / (z1 + z2); c4 = -1.0 * z1 * z2 / r1 / (z1 + z2);
            } else {
                c1 = z2 / r2 / (z1 + z2); c2 = z1 / r1 / (z1 + z2);
                c3 = r2 / (z1 + z2); c4 = -1.0 * r1 / (z1 + z2);
            }
            int no = nidx(K, oc), ns = nidx(K, c);
            flux[0] = kF(uo[no], ro[no], c0, r0, ba) * c1;
            flux[0] += kF(us[ns], rs[ns], c0, r0, ba) * c2;
            flux[0] += kF2(uo[no], ro[no], c0, r0, ba) * c3;
            flux[0] += kF2(us[ns], rs[ns], c0, r0, ba) * c4;
            flux[0] *= -1.;
            for (int m = 0; m < K; m++) {
                c[axis] = m;
                int n = nidx(K, c);
                dR[m] = rs[n];
                vel[m] = us[n];
            }
            /* right face, other = neighbour k+1/j+1/i+1; c[axis] == N here */
            eo = e + st;
            ro = fld(s, src, F_RHO, eo);
            uo = fld(s, src, F_U0 + axis, eo);
            oc[axis] = 0;
            z2 = r0 * c0;
            r2 = r0;
            if (mode == 0) {
                c1 = z2 * r1 / (z1 + z2); c2 = z1 * r2 / (z1 + z2);
                c3 = z1 * z2 / r1 / (z1 + z2); c4 = -1.0 * z1 * z2 / r2 / (z1 + z2);
            } else {
                c1 = z1 / r1 / (z1 + z2); c2 = z2 / r2 / (z1 + z2);
                c3 = r1 / (z1 + z2); c4 = -1.0 * r2 / (z1 + z2);
            }
            no = nidx(K, oc);
            ns = nidx(K, c);
            flux[N] = kF(us[ns], rs[ns], c0, r0, ba) * c1;
            flux[N] += kF(uo[no], ro[no], c0, r0, ba) * c2;
            flux[N] += kF2(us[ns], rs[ns], c0, r0, ba) * c3;
            flux[N] += kF2(uo[no], ro[no], c0, r0, ba) * c4;
            /* volume flux f(line), cppsrc/kernelFuncs.cpp:13-29 */
            for (int m = 0; m < K; m++) {
                if (mode == 0) f[m] = (dR[m] + dR[m] * dR[m] * ba * .5 * (1.0 / r0)) * (c0 * c0 / r0);
                else f[m] = (ba == 0.0) ? vel[m] * r0 : vel[m] * (dR[m] + r0);
            }
            for (int i = 0; i < K; i++) {
                double v = 0;
                for (int k = 0; k < K; k++) v += Sq[i * K + k] * f[k];
                rhs[i] = v - flux[i];
            }
            solve(K, A, rhs, res);
            double* out = fld(s, dst, mode == 0 ? F_U0 + axis : F_RHO, e);
            for (int m = 0; m < K; m++) {
                c[axis] = m;
                out[nidx(K, c)] += res[m];
            }
        }
}

/* Element::OperateQFromDRho (cppsrc/Element.cpp:623-690): LDG gradient with
   central flux, Q_axis = -(M w) \ (S drho + F), written into the SOURCE grid
   (cppsrc/Grid.cpp:667). */
static void op_q_from_drho(dgo_sim* s, grid_t* g, int axis, size_t e)
{
    const int K = s->K, N = s->N;
    const double w = s->p.elem_width[axis];
    const size_t st = ax_stride(s, axis);
    double A[100];
    for (int i = 0; i < K * K; i++) A[i] = w * s->M[i];
    const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
    const double* rs = fld(s, g, F_RHO, e);
    const double* rl = fld(s, g, F_RHO, e - st);
    const double* rr = fld(s, g, F_RHO, e + st);
    double* qd = fld(s, g, F_Q0 + axis, e);
    for (int l1 = 0; l1 < K; l1++)
        for (int l2 = 0; l2 < K; l2++) {
            int c[3], oc[3];
            c[o1] = oc[o1] = l1;
            c[o2] = oc[o2] = l2;
            double flux[10] = {0}, dR[10], rhs[10], res[10];
            c[axis] = 0;
            oc[axis] = N;
            flux[0] = rl[nidx(K, oc)];
            flux[0] += rs[nidx(K, c)];
            flux[0] *= 0.5;
            for (int m = 0; m < K; m++) {
                c[axis] = m;
                dR[m] = rs[nidx(K, c)];
            }
            oc[axis] = 0;
            flux[N] = rs[nidx(K, c)];
            flux[N] += rr[nidx(K, oc)];
            flux[N] *= -0.5;
            for (int i = 0; i < K; i++) {
                double v = 0;
                for (int k = 0; k < K; k++) v += s->S[i * K + k] * dR[k];
                rhs[i] = v + flux[i];
            }
            solve(K, A, rhs, res);
            for (int m = 0; m < K; m++) {
                c[axis] = m;
                qd[nidx(K, c)] = -1.0 * res[m];
            }
        }
}

/* Element::OperateDRhoFromQ (cppsrc/Element.cpp:691-758): drho += (M w) \
   ((S Q + F) * -1 * D), central flux on Q_axis. */
static void op_drho_from_q(dgo_sim* s, grid_t* dst, grid_t* src, int axis, size_t e)
{
    const int K = s->K, N = s->N;
    const double w = s->p.elem_width[axis];
    const double D = s->p.diff_const;
    const size_t st = ax_stride(s, axis);
    double A[100];
    for (int i = 0; i < K * K; i++) A[i] = w * s->M[i];
    const int o1 = (axis + 1) % 3, o2 = (axis + 2) % 3;
    const double* qs = fld(s, src, F_Q0 + axis, e);
    const double* ql = fld(s, src, F_Q0 + axis, e - st);
    const double* qr = fld(s, src, F_Q0 + axis, e + st);
    double* out = fld(s, dst, F_RHO, e);
    for (int l1 = 0; l1 < K; l1++)
        for (int l2 = 0; l2 < K; l2++) {
            int c[3], oc[3];
            c[o1] = oc[o1] = l1;
            c[o2] = oc[o2] = l2;
            double flux[10] = {0}, Q[10], rhs[10], res[10];
            c[axis] = 0;
            oc[axis] = N;
            flux[0] = ql[nidx(K, oc)];
            flux[0] += qs[nidx(K, c)];
            flux[0] *= 0.5;
            for (int m = 0; m < K; m++) {
                c[axis] = m;
                Q[m] = qs[nidx(K, c)];
            }
            oc[axis] = 0;
            flux[N] = qs[nidx(K, c)];
            flux[N] += qr[nidx(K, oc)];
            flux[N] *= -0.5;
            for (int i = 0; i < K; i++) {
                double v = 0;
                for (int k = 0; k < K; k++) v += s->S[i * K + k] * Q[k];
                rhs[i] = ((v + flux[i]) * -1.0) * D;
            }
            solve(K, A, rhs, res);
            for (int m = 0; m < K; m++) {
                c[axis] = m;
                out[nidx(K, c)] += res[m];
            }
        }
}

/* Element::OperateSponge (cppsrc/Element.cpp:760-781). */
static void op_sponge(dgo_sim* s, grid_t* dst, grid_t* src, size_t e)
{
    double sg = s->sigma[e];
    for (int a = 0; a < 3; a++) {
        double* o = fld(s, dst, F_U0 + a, e);
        const double* u = fld(s, src, F_U0 + a, e);
        for (int n = 0; n < s->K3; n++) o[n] += -1.0 * u[n] * sg;
    }
    double* o = fld(s, dst, F_RHO, e);
    const double* r = fld(s, src, F_RHO, e);
    for (int n = 0; n < s->K3; n++) o[n] += -1.0 * r[n] * sg;
}

/* Element::selfWeightedAdd (cppsrc/Element.cpp:288-307), all 7 fields. */
static void self_weighted_add(dgo_sim* s, grid_t* dst, grid_t* other, double a, double b, size_t e)
{
    for (int f = 0; f < NF; f++) {
        double* d = fld(s, dst, f, e);
        const double* o = fld(s, other, f, e);
        for (int n = 0; n < s->K3; n++) d[n] = d[n] * a + o[n] * b;
    }
}

#define FOR_INTERIOR(s, e)                                   \
    for (int _i = 1; _i <= (s)->E[0]; _i++)                  \
        for (int _j = 1; _j <= (s)->E[1]; _j++)              \
            for (int _k = 1; _k <= (s)->E[2]; _k++)          \
                for (size_t e = eidx((s), _i, _j, _k), _once = 1; _once; _once = 0)

/* One RHS application dst += L(src) as one stage of Grid::RK33 does it
   (cppsrc/Grid.cpp:654-704): communicate, LDG (Q into src), communicate,
   divergence, advection per axis (mode 0 then 1), sponge. */
static void stage_rhs(dgo_sim* s, grid_t* dst, grid_t* src, double t_stage)
{
    const dgo_params* p = &s->p;
    communicate(s, src);
    apply_source(s, src, t_stage);
    if (p->eval_diff) {
        FOR_INTERIOR(s, e) for (int a = 0; a < 3; a++) op_q_from_drho(s, src, a, e);
        communicate(s, src);
        FOR_INTERIOR(s, e) for (int a = 0; a < 3; a++) op_drho_from_q(s, dst, src, a, e);
    }
    FOR_INTERIOR(s, e)
    {
        if (p->eval_advect)
            for (int a = 0; a < 3; a++) {
                op_u_from_v(s, dst, src, a, 0, e);
                op_u_from_v(s, dst, src, a, 1, e);
            }
        if (p->eval_sponge) op_sponge(s, dst, src, e);
    }
}

/* Grid::RK33 single-block branch (cppsrc/Grid.cpp:642-834). */
static void rk33(dgo_sim* s, grid_t* self, grid_t* old, grid_t* k1, grid_t* k2, double dt)
{
    const double w23 = s->p.rk_exact ? 2.0 / 3.0 : (double)(2.0f / 3.0f);
    const double w13 = s->p.rk_exact ? 1.0 / 3.0 : (double)(1.0f / 3.0f);
    set_zero(s, k1);
    set_zero(s, k2);
    set_zero(s, self);
    stage_rhs(s, k1, old, s->t);
    FOR_INTERIOR(s, e) self_weighted_add(s, k1, old, dt, 1.0, e);
    stage_rhs(s, k2, k1, s->t + dt);
    FOR_INTERIOR(s, e)
    {
        self_weighted_add(s, k2, k1, dt * .25, .25, e);
        self_weighted_add(s, k2, old, 1.0, .75, e);
    }
    stage_rhs(s, self, k2, s->t + 0.5 * dt);
    FOR_INTERIOR(s, e)
    {
        self_weighted_add(s, self, k2, dt * 2.0 / 3.0, w23, e);
        self_weighted_add(s, self, old, 1.0, w13, e);
    }
}

dgo_sim* dgo_create(const dgo_params* p, const double* mass_m, const double* stiff,
                    const double* zeros)
{
    if (p->order < 1 || p->order > 9) return NULL;
    dgo_sim* s = (dgo_sim*)calloc(1, sizeof(dgo_sim));
    s->p = *p;
    s->N = p->order;
    s->K = p->order + 1;
    s->K3 = s->K * s->K * s->K;
    for (int a = 0; a < 3; a++) {
        s->E[a] = p->num_elements[a] * p->num_blocks[a];
        s->H[a] = s->E[a] + 2;
    }
    s->nelh = (size_t)s->H[0] * s->H[1] * s->H[2];
    memcpy(s->M, mass_m, sizeof(double) * s->K * s->K);
    memcpy(s->S, stiff, sizeof(double) * s->K * s->K);
    memcpy(s->zeros, zeros, sizeof(double) * s->K);
    for (int i = 0; i < 4; i++) {
        s->g[i].f = (double*)calloc((size_t)NF * s->nelh * s->K3, sizeof(double));
        if (!s->g[i].f) { dgo_destroy(s); return NULL; }
    }
    s->sigma = (double*)calloc(s->nelh, sizeof(double));
    s->coords = (double*)calloc((size_t)3 * s->nelh * s->K3, sizeof(double));

    /* Geometry and IC: cppsrc/Block.cpp:167-247 (element corners from the
       block corner, sigma from the nearest sponged face), cppsrc/Element.cpp:
       166-189 (node coordinates), cppsrc/Node.cpp:76-100 (Gaussian IC, also in
       halo elements). */
    const int K = s->K;
    double dist[6] = {1e9, 1e9, 1e9, 1e9, 1e9, 1e9};
    for (int i = 0; i < s->H[0]; i++)
        for (int j = 0; j < s->H[1]; j++)
            for (int k = 0; k < s->H[2]; k++) {
                int gpos[3] = {i - 1, j - 1, k - 1};
                double ecorner[3];
                for (int a = 0; a < 3; a++) {
                    int E = p->num_elements[a];
                    int b = gpos[a] < 0 ? 0 : (gpos[a] >= s->E[a] ? p->num_blocks[a] - 1 : gpos[a] / E);
                    int li = gpos[a] - b * E + 1;
                    double bc = p->corner[a] + p->elem_width[a] * E * b;
                    ecorner[a] = (li - 1) * p->elem_width[a] + bc;
                }
                for (int a = 0; a < 3; a++) {
                    if (p->sponge_width[2 * a] > 0) dist[2 * a] = abs(gpos[a]) * p->elem_width[a];
                    if (p->sponge_width[2 * a + 1] > 0)
                        dist[2 * a + 1] = abs(s->E[a] - abs(gpos[a]) - 1) * p->elem_width[a];
                }
                int edge = 0;
                double sh = dist[0];
                for (int t = 1; t < 6; t++)
                    if (dist[t] < sh) { edge = t; sh = dist[t]; }
                sh /= (double)p->sponge_width[edge] * p->elem_width[edge / 2];
                size_t e = eidx(s, i, j, k);
                s->sigma[e] = p->sponge_width[edge] == 0 ? 0.0 : fmax(0.0, 1.0 - sh) * p->sigma_max;
                for (int a0 = 0; a0 < K; a0++)
                    for (int a1 = 0; a1 < K; a1++)
                        for (int a2 = 0; a2 < K; a2++) {
                            int c[3] = {a0, a1, a2};
                            int n = nidx(K, c);
                            double x[3];
                            for (int a = 0; a < 3; a++) {
                                x[a] = p->elem_width[a] * (zeros[c[a]] / 2.0 + .5) + ecorner[a];
                                s->coords[((size_t)a * s->nelh + e) * s->K3 + n] = x[a];
                            }
                            if (p->ic_gauss[0] || p->ic_gauss[1] || p->ic_gauss[2]) {
                                double d2 = 0;
                                for (int a = 0; a < 3; a++)
                                    if (p->ic_gauss[a]) d2 += (x[a] - p->ic_center[a]) * (x[a] - p->ic_center[a]);
                                double d = sqrt(d2);
                                double g = exp(-(d) * (d) / (1.0 / p->ic_sigma));
                                fld(s, &s->g[0], F_RHO, e)[n] = p->ic_drho_amp * g;
                                for (int a = 0; a < 3; a++)
                                    fld(s, &s->g[0], F_U0 + a, e)[n] = p->ic_v_amp[a] * exp(-(d) * (d) / (1.0 / p->ic_sigma));
                            }
                        }
            }
    for (int i = 1; i < 4; i++) memcpy(s->g[i].f, s->g[0].f, sizeof(double) * NF * s->nelh * s->K3);
    s->cur = 1; /* newGrid = &myGrid2 (cppsrc/driver.cpp:216) */
    s->t = 0.0;
    return s;
}

void dgo_destroy(dgo_sim* s)
{
    if (!s) return;
    for (int i = 0; i < 4; i++) free(s->g[i].f);
    free(s->sigma);
    free(s->coords);
    free(s);
}

/* The driver's step loop (cppsrc/driver.cpp:256-277): swap, RK33, t += dt. */
void dgo_run(dgo_sim* s, double dt, int nsteps)
{
    for (int n = 0; n < nsteps; n++) {
        int old = s->cur;
        int nw = old == 1 ? 0 : 1;
        rk33(s, &s->g[nw], &s->g[old], &s->g[2], &s->g[3], dt);
        s->cur = nw;
        s->t += dt;
    }
}

static void gather(const dgo_sim* s, const grid_t* g, int f, double* out)
{
    const int K = s->K;
    const size_t X = (size_t)s->E[0] * K, Y = (size_t)s->E[1] * K, Z = (size_t)s->E[2] * K;
    for (size_t ii = 0; ii < X; ii++)
        for (size_t jj = 0; jj < Y; jj++)
            for (size_t kk = 0; kk < Z; kk++) {
                size_t e = eidx(s, (int)(ii / K) + 1, (int)(jj / K) + 1, (int)(kk / K) + 1);
                int c[3] = {(int)(ii % K), (int)(jj % K), (int)(kk % K)};
                out[(ii * Y + jj) * Z + kk] = fld(s, g, f, e)[nidx(K, c)];
            }
}

static void scatter(dgo_sim* s, grid_t* g, int f, const double* in)
{
    const int K = s->K;
    const size_t X = (size_t)s->E[0] * K, Y = (size_t)s->E[1] * K, Z = (size_t)s->E[2] * K;
    for (size_t ii = 0; ii < X; ii++)
        for (size_t jj = 0; jj < Y; jj++)
            for (size_t kk = 0; kk < Z; kk++) {
                size_t e = eidx(s, (int)(ii / K) + 1, (int)(jj / K) + 1, (int)(kk / K) + 1);
                int c[3] = {(int)(ii % K), (int)(jj % K), (int)(kk % K)};
                fld(s, g, f, e)[nidx(K, c)] = in[(ii * Y + jj) * Z + kk];
            }
}

void dgo_get_state(const dgo_sim* s, double* rho, double* vel)
{
    size_t n = (size_t)s->E[0] * s->E[1] * s->E[2] * s->K3;
    gather(s, &s->g[s->cur], F_RHO, rho);
    for (int a = 0; a < 3; a++) gather(s, &s->g[s->cur], F_U0 + a, vel + a * n);
}

void dgo_set_state(dgo_sim* s, const double* rho, const double* vel)
{
    size_t n = (size_t)s->E[0] * s->E[1] * s->E[2] * s->K3;
    set_zero(s, &s->g[s->cur]);
    scatter(s, &s->g[s->cur], F_RHO, rho);
    for (int a = 0; a < 3; a++) scatter(s, &s->g[s->cur], F_U0 + a, vel + a * n);
}

void dgo_get_coords(const dgo_sim* s, double* coords, double* sigma)
{
    const int K = s->K;
    const size_t X = (size_t)s->E[0] * K, Y = (size_t)s->E[1] * K, Z = (size_t)s->E[2] * K;
    const size_t n = X * Y * Z;
    for (size_t ii = 0; ii < X; ii++)
        for (size_t jj = 0; jj < Y; jj++)
            for (size_t kk = 0; kk < Z; kk++) {
                size_t e = eidx(s, (int)(ii / K) + 1, (int)(jj / K) + 1, (int)(kk / K) + 1);
                int c[3] = {(int)(ii % K), (int)(jj % K), (int)(kk % K)};
                size_t p = (ii * Y + jj) * Z + kk;
                for (int a = 0; a < 3; a++)
                    coords[a * n + p] = s->coords[((size_t)a * s->nelh + e) * s->K3 + nidx(K, c)];
                if (sigma) sigma[p] = s->sigma[e];
            }
}

double dgo_time(const dgo_sim* s) { return s->t; }

void dgo_rhs(dgo_sim* s, double* rho, double* vel)
{
    grid_t* src = &s->g[s->cur];
    grid_t* dst = &s->g[2];
    size_t n = (size_t)s->E[0] * s->E[1] * s->E[2] * s->K3;
    set_zero(s, dst);
    stage_rhs(s, dst, src, s->t);
    gather(s, dst, F_RHO, rho);
    for (int a = 0; a < 3; a++) gather(s, dst, F_U0 + a, vel + a * n);
}
