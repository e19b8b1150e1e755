/*
 * oracle_body.h — precision-generic part of the oracle (TEST INFRASTRUCTURE ONLY, see asph_oracle.h).
 * Included three times by asph_oracle.c: REAL=float on the FP32 state (the canonical mirror, suffix f32),
 * REAL=double on the FP32 state (FP64 arithmetic on the GPU's inputs, suffix f64) and REAL=double on the FP64 state
 * of the FP64 step (suffix d64). Requires: REAL, F(name), FMA, SQRT, WCOEF, DCOEF; STATE and SREAL (the state struct
 * and its element type), ITPOS(p, tmp) (a float pointer to the position p for the cell iterator) and
 * SUM_KIND(g, s, c, i) (how a particle's sums are dealt to lanes; always sequential on the FP64 state).
 *
 * Formulas (reference file:line):
 *   Wendland C2 kernel and derivative ........ cuda/src/algorithm/WendlandKernel.cuh:39-52, 69-84
 *   Tait equation of state, gamma = 5 ........ cuda/src/algorithm/Common.cuh:6-12
 *   density ................................... cuda/src/algorithm/Algorithm.cu:17-54
 *   boundary density .......................... cuda/src/algorithm/BoundaryAlgorithm.cu:15-51
 *   gravity / pressure / viscosity / cohesion . cuda/src/algorithm/Algorithm.cu:56-232
 *   boundary pressure / friction .............. cuda/src/algorithm/BoundaryAlgorithm.cu:53-162
 *
 * Canonical operation order (shared with the CUDA kernels, documented where it departs from the
 * reference): squared distances are fma(dz,dz,fma(dy,dy,dx*dx)); q = r * (1/h) instead of r / h;
 * the kernel prefactors coef/h^3 and dcoef/h^4 are formed once per particle; the Tait pressure is
 * B*d*(5+d*(10+d*(10+d*(5+d)))) with d = (rho-rho0)/rho0, algebraically (rho/rho0)^5-1 without
 * the cancellation of powf(...)-1; directions are offset * (1/r); per-pair force terms are a scalar
 * s times the direction, accumulated with fma.
 *
 * Summation order (sum_kind): neighbours are summed in the canonical visiting order of the candidate cells. Three
 * kinds of particles are summed as the GPU sums them with one warp, each lane summing its share in the canonical
 * order and the 32 partial sums combined by the butterfly s_l <- s_l + s_(l xor o) for o = 16, 8, 4, 2, 1:
 *   - a particle whose query box spans more than ORC_HEAVY_CELLS reference cells ("heavy", after merges made h
 *     large), or whose neighbour-list row would need more than ORC_LIST_ENTRIES entries: the box's sub-cell with
 *     canonical index t (see orc_iter.t) goes to lane t mod 32;
 *   - a particle whose row has more than ORC_ROW_HEAVY entries (many neighbours): row entry e goes to lane e mod 32.
 * Their boundary terms are dealt by member: member k of each visited boundary cell (counted from the cell's first
 * member) goes to lane k mod 32.
 */

/* W(r, h) with precomputed 1/h and coef/h^3 */
static inline REAL F(kernel_w)(REAL r, REAL invh, REAL wc)
{
    const REAL q = r * invh;
    if (q > (REAL)2) {
        return (REAL)0;
    }
    const REAL t = FMA((REAL)-0.5, q, (REAL)1);
    const REAL t2 = t * t;
    return (wc * (t2 * t2)) * FMA((REAL)2, q, (REAL)1);
}

/* dW/dr(r, h) with precomputed 1/h and dcoef/h^4 */
static inline REAL F(kernel_dw)(REAL r, REAL invh, REAL dwc)
{
    const REAL q = r * invh;
    if (q > (REAL)2) {
        return (REAL)0;
    }
    const REAL t = FMA((REAL)-0.5, q, (REAL)1);
    const REAL t3 = (t * t) * t;
    return (dwc * q) * t3;
}

static inline void F(kernel_consts)(REAL h, REAL* invh, REAL* wc, REAL* dwc)
{
    const REAL h3 = (h * h) * h;
    *invh = (REAL)1 / h;
    *wc = WCOEF / h3;
    *dwc = DCOEF / (h3 * h);
}

/* p / rho^2 with the Tait equation (Common.cuh:6-12) */
static inline REAL F(pressure_term)(REAL rho, REAL rho0, REAL c0)
{
    const REAL B = ((rho0 * c0) * c0) / (REAL)5;
    const REAL d = (rho - rho0) / rho0;
    REAL u = (REAL)5 + d;
    u = FMA(d, u, (REAL)10);
    u = FMA(d, u, (REAL)10);
    u = FMA(d, u, (REAL)5);
    const REAL p = B * (d * u);
    return p / (rho * rho);
}

/* neighbour coordinate a of p, shifted by the periodic image offset of its cell (sh) */
#define NBR(p, a) (g->periodic ? (REAL)(p)[a] + (REAL)sh[a] : (REAL)(p)[a])

static inline REAL F(dist2)(REAL dx, REAL dy, REAL dz)
{
    return FMA(dz, dz, FMA(dy, dy, dx * dx));
}

/* the warp's combination of 32 partial sums */
static REAL F(butterfly)(REAL* s)
{
    REAL t[ORC_LANES];
    for (int o = ORC_LANES / 2; o >= 1; o >>= 1) {
        for (int l = 0; l < ORC_LANES; l++) {
            t[l] = s[l] + s[l ^ o];
        }
        memcpy(s, t, sizeof(t));
    }
    return s[0];
}

/* Fluid part of the density of particle i into out[lanes]. The members of each visited sub-cell are taken in blocks
 * of up to 32 (the blocks of the neighbour-list row, see list_entries). deal = ORC_DEAL_SUBCELL: the box's sub-cell
 * t goes to lane t mod lanes; ORC_DEAL_ENTRY: the e-th block holding an accepted neighbour (row entry e) goes to
 * lane e mod lanes; lanes = 1 is the sequential sum. */
static void F(density_fluid)(const orc_grid* g, const STATE* s, const orc_cells* c, int64_t i, int deal,
                             int lanes, REAL* out)
{
    const SREAL* pi = s->pos + 4 * i;
    const REAL xi = pi[0], yi = pi[1], zi = pi[2];
    const float R = (float)(s->h[i] + s->h[i]);
    float pif[4];
    for (int l = 0; l < lanes; l++) {
        out[l] = 0;
    }
    uint32_t e = 0;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    it_init(&it, g, c->start, c->end, c->ex, ITPOS(pi, pif), R);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t blk0 = jb; blk0 < je; blk0 += 32) {
            const uint32_t blk1 = je - blk0 < 32u ? je : blk0 + 32u;
            REAL* rho = out + (deal == ORC_DEAL_ENTRY ? e : it.t) % (uint32_t)lanes;
            int any = 0;
            for (uint32_t j = blk0; j < blk1; j++) {
                const SREAL* pj = s->pos + 4 * (size_t)j;
                const REAL dx = NBR(pj, 0) - xi;
                const REAL dy = NBR(pj, 1) - yi;
                const REAL dz = NBR(pj, 2) - zi;
                const REAL r2 = F(dist2)(dx, dy, dz);
                const REAL hj = s->h[j];
                const REAL twoh = hj + hj;
                if (r2 > twoh * twoh) {
                    continue;
                }
                any = 1;
                REAL invh, wc, dwc;
                F(kernel_consts)(hj, &invh, &wc, &dwc);
                const REAL w = F(kernel_w)(SQRT(r2), invh, wc);
                *rho = FMA((REAL)s->m[j], w, *rho);
            }
            e += (uint32_t)any;
        }
    }
}

/* boundary part of the density into out[lanes]: member k of each boundary cell (counted from its first member) on
 * lane k mod lanes */
static void F(density_boundary)(const orc_grid* g, const STATE* s, const orc_boundary* b, int64_t i,
                                int lanes, REAL* out)
{
    for (int l = 0; l < lanes; l++) {
        out[l] = 0;
    }
    if (b == NULL || b->n == 0) {
        return;
    }
    const SREAL* pi = s->pos + 4 * i;
    const REAL xi = pi[0], yi = pi[1], zi = pi[2];
    const REAL hi = s->h[i];
    const float R = (float)(s->h[i] + s->h[i]);
    float pif[4];
    REAL invh, wc, dwc;
    F(kernel_consts)(hi, &invh, &wc, &dwc);
    const REAL twoh = hi + hi;
    const REAL cut = twoh * twoh;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    it_init(&it, g, b->start, b->end, b->ex, ITPOS(pi, pif), R);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t k = jb; k < je; k++) {
            REAL* rb = out + (k - jb) % (uint32_t)lanes;
            const float* pb = b->pos + 4 * (size_t)k;
            const REAL dx = NBR(pb, 0) - xi;
            const REAL dy = NBR(pb, 1) - yi;
            const REAL dz = NBR(pb, 2) - zi;
            const REAL r2 = F(dist2)(dx, dy, dz);
            if (r2 > cut) {
                continue;
            }
            const REAL w = F(kernel_w)(SQRT(r2), invh, wc);
            *rb = FMA((REAL)b->psi[k], w, *rb);
        }
    }
}

void F(orc_density_impl)(const orc_grid* g, const orc_params* P, const STATE* s, const orc_cells* c,
                         const orc_boundary* b, REAL* rho_out)
{
    (void)P;
    const int64_t n = s->n;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
        REAL rho, rb;
        const int deal = SUM_KIND(g, s, c, i);
        if (deal != ORC_DEAL_NONE) {
            REAL pf[ORC_LANES], pb[ORC_LANES];
            F(density_fluid)(g, s, c, i, deal, ORC_LANES, pf);
            F(density_boundary)(g, s, b, i, ORC_LANES, pb);
            rho = F(butterfly)(pf);
            rb = F(butterfly)(pb);
        } else {
            F(density_fluid)(g, s, c, i, ORC_DEAL_NONE, 1, &rho);
            F(density_boundary)(g, s, b, i, 1, &rb);
        }
        rho_out[i] = rho + rb;
    }
}

/* accumulators of the force pass: pressure, viscosity, cohesion; boundary pressure, boundary friction */
typedef struct F(facc) {
    REAL ap[3], av[3], as[3], bp[3], bf[3];
    double scale;
} F(facc);

/* force terms of particle i into fl[lanes], the fluid blocks dealt as in density_fluid, boundary member k of each
 * boundary cell on lane k mod lanes */
static void F(forces_part)(const orc_grid* g, const orc_params* P, const STATE* s, const orc_cells* c,
                           const orc_boundary* b, const SREAL* rho_in, int64_t i, int deal, int lanes, F(facc) * fl)
{
    const REAL rho0 = P->rho0, c0 = P->c0;
    const REAL alpha = P->alpha, nu_k = P->nu;
    const int morris = P->viscosity_model == 1u;
    const int visc_on = morris ? (P->nu != 0.0f) : (P->alpha != 0.0f);
    const int sigma_on = P->sigma != 0.0f;
    const SREAL* pi = s->pos + 4 * i;
    const SREAL* vi4 = s->vel + 4 * i;
    const REAL xi = pi[0], yi = pi[1], zi = pi[2];
    const REAL vxi = vi4[0], vyi = vi4[1], vzi = vi4[2];
    const REAL hi = s->h[i], mi = s->m[i];
    const REAL rhoi = rho_in[i];
    const REAL pti = F(pressure_term)(rhoi, rho0, c0);
    const REAL Ki = (((REAL)2 * alpha) * hi) * c0;
    const REAL ei = ((REAL)0.01 * hi) * hi;
    const float R = (float)(s->h[i] + s->h[i]);
    float pif[4];
    memset(fl, 0, sizeof(*fl) * (size_t)lanes);
    uint32_t e = 0;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    it_init(&it, g, c->start, c->end, c->ex, ITPOS(pi, pif), R);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t blk0 = jb; blk0 < je; blk0 += 32) {
            const uint32_t blk1 = je - blk0 < 32u ? je : blk0 + 32u;
            F(facc)* f = fl + (deal == ORC_DEAL_ENTRY ? e : it.t) % (uint32_t)lanes;
            int any = 0;
            for (uint32_t j = blk0; j < blk1; j++) {
                if ((int64_t)j == i) {
                    any = 1; /* the particle itself is accepted (its row holds it) but adds no force */
                    continue;
                }
                const SREAL* pj = s->pos + 4 * (size_t)j;
                const REAL dx = xi - NBR(pj, 0);
                const REAL dy = yi - NBR(pj, 1);
                const REAL dz = zi - NBR(pj, 2);
                const REAL r2 = F(dist2)(dx, dy, dz);
                const REAL hj = s->h[j];
                const REAL twoh = hj + hj;
                if (r2 > twoh * twoh) {
                    continue;
                }
                any = 1;
                REAL invh, wc, dwc;
                F(kernel_consts)(hj, &invh, &wc, &dwc);
                const REAL r = SQRT(r2);
                REAL u[3];
                if (r > (REAL)0) {
                    const REAL ir = (REAL)1 / r;
                    u[0] = dx * ir;
                    u[1] = dy * ir;
                    u[2] = dz * ir;
                } else {
                    u[0] = 0;
                    u[1] = 1;
                    u[2] = 0;
                }
                const REAL dw = F(kernel_dw)(r, invh, dwc);
                const REAL mj = s->m[j];
                const REAL rhoj = rho_in[j];
                const REAL ptj = F(pressure_term)(rhoj, rho0, c0);
                {
                    const REAL sp = (mj * dw) * (pti + ptj);
                    for (int a = 0; a < 3; a++) {
                        f->ap[a] = FMA(-sp, u[a], f->ap[a]);
                    }
                    f->scale += fabs((double)sp);
                }
                if (visc_on) {
                    const SREAL* vj4 = s->vel + 4 * (size_t)j;
                    const REAL vd[3] = {vxi - (REAL)vj4[0], vyi - (REAL)vj4[1], vzi - (REAL)vj4[2]};
                    if (!morris) {
                        const REAL comp = FMA(vd[2], dz, FMA(vd[1], dy, vd[0] * dx));
                        if (comp < (REAL)0) {
                            const REAL nuij = Ki / (rhoi + rhoj);
                            const REAL piv = (-nuij * comp) / (r2 + ei);
                            const REAL sv = (mj * piv) * dw;
                            for (int a = 0; a < 3; a++) {
                                f->av[a] = FMA(-sv, u[a], f->av[a]);
                            }
                            f->scale += fabs((double)sv);
                        }
                    } else {
                        const REAL coef = ((mj * nu_k) * (rhoi + rhoj)) / (rhoi * rhoj);
                        const REAL sv = coef * ((r * dw) / (r2 + ei));
                        for (int a = 0; a < 3; a++) {
                            f->av[a] = FMA(sv, vd[a], f->av[a]);
                        }
                        f->scale +=
                            fabs((double)sv) * sqrt((double)vd[0] * vd[0] + (double)vd[1] * vd[1] + (double)vd[2] * vd[2]);
                    }
                }
                if (sigma_on) {
                    const REAL ss = mj * F(kernel_w)(r, invh, wc);
                    for (int a = 0; a < 3; a++) {
                        f->as[a] = FMA(ss, u[a], f->as[a]);
                    }
                    f->scale += fabs((double)((REAL)P->sigma / mi) * (double)ss);
                }
            }
            e += (uint32_t)any;
        }
    }
    if (b != NULL && b->n > 0) {
        REAL invh, wc, dwc;
        F(kernel_consts)(hi, &invh, &wc, &dwc);
        const REAL twoh = hi + hi;
        const REAL cut = twoh * twoh;
        it_init(&it, g, b->start, b->end, b->ex, ITPOS(pi, pif), R);
        while (it_next(&it, &jb, &je, sh)) {
            for (uint32_t k = jb; k < je; k++) {
                F(facc)* f = fl + (k - jb) % (uint32_t)lanes;
                const float* pb = b->pos + 4 * (size_t)k;
                const REAL dx = xi - NBR(pb, 0);
                const REAL dy = yi - NBR(pb, 1);
                const REAL dz = zi - NBR(pb, 2);
                const REAL r2 = F(dist2)(dx, dy, dz);
                if (r2 > cut) {
                    continue;
                }
                const REAL r = SQRT(r2);
                REAL u[3];
                if (r > (REAL)0) {
                    const REAL ir = (REAL)1 / r;
                    u[0] = dx * ir;
                    u[1] = dy * ir;
                    u[2] = dz * ir;
                } else {
                    u[0] = 0;
                    u[1] = 1;
                    u[2] = 0;
                }
                const REAL dw = F(kernel_dw)(r, invh, dwc);
                const REAL psi = b->psi[k];
                const REAL sp = (psi * pti) * dw;
                for (int a = 0; a < 3; a++) {
                    f->bp[a] = FMA(-sp, u[a], f->bp[a]);
                }
                f->scale += fabs((double)sp);
                const REAL comp = FMA(vzi, dz, FMA(vyi, dy, vxi * dx));
                if (comp < (REAL)0) {
                    const REAL nub = (((REAL)b->fric[k] * hi) * c0) / ((REAL)2 * rhoi);
                    const REAL pib = (-nub * comp) / (r2 + ei);
                    const REAL sf = (psi * pib) * dw;
                    for (int a = 0; a < 3; a++) {
                        f->bf[a] = FMA(-sf, u[a], f->bf[a]);
                    }
                    f->scale += fabs((double)sf);
                }
            }
        }
    }
}

/* Force pass. rho: densities of the state (FP32 values, as the GPU holds them). */
void F(orc_forces_impl)(const orc_grid* g, const orc_params* P, const STATE* s, const orc_cells* c,
                        const orc_boundary* b, const SREAL* rho_in, REAL* acc_out, double* scale_out)
{
    const int64_t n = s->n;
    const int morris = P->viscosity_model == 1u;
    const int visc_on = morris ? (P->nu != 0.0f) : (P->alpha != 0.0f);
    const int sigma_on = P->sigma != 0.0f;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
        F(facc) f;
        const int deal = SUM_KIND(g, s, c, i);
        if (deal != ORC_DEAL_NONE) {
            F(facc) part[ORC_LANES];
            F(forces_part)(g, P, s, c, b, rho_in, i, deal, ORC_LANES, part);
            memset(&f, 0, sizeof(f));
            REAL t[ORC_LANES];
#define ORC_REDUCE(field, a)                       \
    for (int l = 0; l < ORC_LANES; l++) {          \
        t[l] = part[l].field[a];                   \
    }                                              \
    f.field[a] = F(butterfly)(t);
            for (int a = 0; a < 3; a++) {
                ORC_REDUCE(ap, a)
                ORC_REDUCE(av, a)
                ORC_REDUCE(as, a)
                ORC_REDUCE(bp, a)
                ORC_REDUCE(bf, a)
            }
#undef ORC_REDUCE
            for (int l = 0; l < ORC_LANES; l++) {
                f.scale += part[l].scale;
            }
        } else {
            F(forces_part)(g, P, s, c, b, rho_in, i, ORC_DEAL_NONE, 1, &f);
        }
        REAL ax = P->gravity[0], ay = P->gravity[1], az = P->gravity[2];
        ax = ax + f.ap[0];
        ay = ay + f.ap[1];
        az = az + f.ap[2];
        if (visc_on) {
            ax = ax + f.av[0];
            ay = ay + f.av[1];
            az = az + f.av[2];
        }
        if (sigma_on) {
            const REAL fs = (REAL)P->sigma / (REAL)s->m[i];
            ax = ax + fs * f.as[0];
            ay = ay + fs * f.as[1];
            az = az + fs * f.as[2];
        }
        ax = ax + f.bp[0];
        ay = ay + f.bp[1];
        az = az + f.bp[2];
        ax = ax + f.bf[0];
        ay = ay + f.bf[1];
        az = az + f.bf[2];
        acc_out[4 * i + 0] = ax;
        acc_out[4 * i + 1] = ay;
        acc_out[4 * i + 2] = az;
        acc_out[4 * i + 3] = 0;
        if (scale_out != NULL) {
            const double g2 = (double)P->gravity[0] * P->gravity[0] + (double)P->gravity[1] * P->gravity[1] +
                              (double)P->gravity[2] * P->gravity[2];
            scale_out[i] = f.scale + sqrt(g2);
        }
    }
}
