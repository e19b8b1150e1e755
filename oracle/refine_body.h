/*
 * refine_body.h — precision-generic refinement pass of the oracle (TEST INFRASTRUCTURE ONLY, see asph_oracle.h).
 * Included twice by asph_oracle.c: on the FP32 state in the canonical FP32 arithmetic (suffix f32, the bit-exact
 * checker of the CUDA refinement kernels) and on the FP64 state in double arithmetic (suffix d64, the refinement of
 * the FP64 step). Requires the macros of oracle_body.h plus CBRT (cube root), PI_R (pi in REAL), SORTABLE(x) and
 * SORTABLE_DESC(x) (uint64 keys ordering scores ascending / descending), and the types orc_sel, cmp_sel.
 * Decisions that the reference takes in FP32 on its parameters (the batch limit round(N * maxBatchRatio)) stay in
 * FP32 in both variants.
 */
/* checkIfParticleCanBeSplitInsideDomain (cuda/src/simulation/refinement/criteria/Common.cuh:6-20) */
static int F(inside_domain)(const orc_params* P, const REAL* p, REAL h, REAL eps)
{
    const REAL mo = eps * h;
    if (p[0] - mo < P->dmin[0] || p[0] + mo > P->dmax[0] || p[1] - mo < P->dmin[1] || p[1] + mo > P->dmax[1] ||
        p[2] - mo < P->dmin[2] || p[2] + mo > P->dmax[2]) {
        return 0;
    }
    return 1;
}

/* velocity-gradient sum of VorticityCriterion.cuh:198-229 (search radius h_i); returns |curl v| or -1 when
 * fewer than 4 neighbours qualify */
static REAL F(vorticity_mag)(const orc_grid* g, const STATE* s, const orc_cells* c, uint32_t i)
{
    const REAL* pi = s->pos + 4 * (size_t)i;
    const REAL* vi = s->vel + 4 * (size_t)i;
    const REAL hi = s->h[i];
    REAL invh, wc, dwc;
    F(kernel_consts)(hi, &invh, &wc, &dwc);
    REAL d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int valid = 0;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    float pif[4];
    it_init(&it, g, c->start, c->end, c->ex, ITPOS(pi, pif), (float)hi);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t j = jb; j < je; j++) {
            if (j == i) {
                continue;
            }
            const REAL* pj = s->pos + 4 * (size_t)j;
            const REAL rx = pj[0] - pi[0], ry = pj[1] - pi[1], rz = pj[2] - pi[2];
            const REAL dist = SQRT(FMA(rz, rz, FMA(ry, ry, rx * rx)));
            if (dist < hi && dist > 1e-6f) {
                const REAL* vj = s->vel + 4 * (size_t)j;
                const REAL vd[3] = {vj[0] - vi[0], vj[1] - vi[1], vj[2] - vi[2]};
                const REAL gw = F(kernel_dw)(dist, invh, dwc);
                const REAL w = s->m[j] / s->rho[j];
                const REAL gd[3] = {rx / dist, ry / dist, rz / dist};
                for (int a = 0; a < 3; a++) {
                    for (int bb = 0; bb < 3; bb++) {
                        d[3 * a + bb] = FMA((w * vd[a]) * gd[bb], gw, d[3 * a + bb]);
                    }
                }
                valid++;
            }
        }
    }
    if (valid < 4) {
        return -1.0f;
    }
    /* d[3a+b] = dv_a/dx_b ; omega = (dvz/dy - dvy/dz, dvx/dz - dvz/dx, dvy/dx - dvx/dy) */
    const REAL ox = d[7] - d[5], oy = d[2] - d[6], oz = d[3] - d[1];
    return SQRT(FMA(oz, oz, FMA(oy, oy, ox * ox)));
}

/* calculateMinSurfaceDistance (InterfaceCriterion.cuh:52-67) */
static void F(min_surface_distance)(const orc_params* P, const REAL* p, REAL out[3])
{
    for (int a = 0; a < 3; a++) {
        const REAL lo = p[a] - P->dmin[a];
        const REAL hi = P->dmax[a] - p[a];
        const REAL m = hi < lo ? hi : lo;
        out[a] = m < 0.0f ? 0.0f : m;
    }
}

static REAL F(compmin3)(const REAL v[3])
{
    REAL m = v[0];
    m = v[1] < m ? v[1] : m;
    m = v[2] < m ? v[2] : m;
    return m;
}

/* Neighbour-count deficit of the free-surface criterion (no reference counterpart): N = #{j != i : r^2 <= (2 h_j)^2}
 * over the candidate cells of [x - 2h_i, x + 2h_i] (the count of sumAllNeighbors, Algorithm.cu:234-268), against
 * N_ref = (4 pi / 3) (2 h_i)^3 rho0 / m_i - 1; returns 1 - N / N_ref. */
static REAL F(neighbour_deficit)(const orc_grid* g, const orc_params* P, const STATE* s, const orc_cells* c,
                                 uint32_t i)
{
    const REAL* pi = s->pos + 4 * (size_t)i;
    const REAL xi = pi[0], yi = pi[1], zi = pi[2];
    const REAL R2 = s->h[i] + s->h[i];
    uint32_t cnt = 0;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    float pif[4];
    it_init(&it, g, c->start, c->end, c->ex, ITPOS(pi, pif), (float)R2);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t j = jb; j < je; j++) {
            if (j == i) {
                continue;
            }
            const SREAL* pj = s->pos + 4 * (size_t)j;
            const REAL dx = NBR(pj, 0) - xi;
            const REAL dy = NBR(pj, 1) - yi;
            const REAL dz = NBR(pj, 2) - zi;
            const REAL r2 = F(dist2)(dx, dy, dz);
            const REAL twoh = s->h[j] + s->h[j];
            cnt += r2 <= twoh * twoh;
        }
    }
    const REAL nref = (((REAL)ORC_FOUR_THIRDS_PI * ((R2 * R2) * R2)) * (REAL)P->rho0) / s->m[i] - (REAL)1;
    return (REAL)1 - (REAL)cnt / nref;
}

/* merge criterion generators: VelocityCriterion.cuh:208-227, InterfaceCriterion.cuh:97-115,
 * VorticityCriterion.cuh:248-312; free surface (3): see neighbour_deficit */
static REAL F(merge_score)(const orc_grid* g, const orc_params* P, const orc_refine* R, const STATE* s,
                         const orc_cells* c, uint32_t i, REAL maxMass)
{
    if (s->m[i] > maxMass) {
        return -1.0f;
    }
    const REAL* p = s->pos + 4 * (size_t)i;
    if (R->criterion == 1u) {
        REAL md[3], nd[3];
        F(min_surface_distance)(P, p, md);
        for (int a = 0; a < 3; a++) {
            nd[a] = md[a] / (R->iface_merge * (P->dmax[a] - P->dmin[a]));
        }
        return F(compmin3)(nd) - 1.0f;
    }
    if (R->criterion == 2u) {
        const REAL mag = F(vorticity_mag)(g, s, c, i);
        if (mag < 0.0f) {
            return -1.0f;
        }
        if (mag < R->vort_merge) {
            return mag / R->vort_merge;
        }
        return -1.0f;
    }
    if (R->criterion == 3u) {
        const REAL d = F(neighbour_deficit)(g, P, s, c, i);
        const REAL t = R->fs_merge;
        return d <= t ? ((d > (REAL)0 ? d : (REAL)0) + t) / (t + t) : (REAL)-1;
    }
    const REAL* v = s->vel + 4 * (size_t)i;
    const REAL sp = SQRT(FMA(v[2], v[2], FMA(v[1], v[1], v[0] * v[0])));
    if (sp < R->vel_merge) {
        return sp / R->vel_merge;
    }
    return -1.0f;
}

/* split criterion generators: VelocityCriterion.cuh:180-206, InterfaceCriterion.cuh:69-95,
 * VorticityCriterion.cuh:170-246 */
static REAL F(split_score)(const orc_grid* g, const orc_params* P, const orc_refine* R, const STATE* s,
                         const orc_cells* c, uint32_t i, REAL minMass)
{
    if (s->m[i] < minMass) {
        return -1.0f;
    }
    const REAL* p = s->pos + 4 * (size_t)i;
    const REAL h = s->h[i];
    if (R->criterion == 1u) {
        REAL md[3], nd[3];
        F(min_surface_distance)(P, p, md);
        if (F(compmin3)(md) < R->eps * h) {
            return -1.0f;
        }
        for (int a = 0; a < 3; a++) {
            nd[a] = md[a] / (R->iface_split * (P->dmax[a] - P->dmin[a]));
        }
        return 1.0f - F(compmin3)(nd);
    }
    if (!F(inside_domain)(P, p, h, R->eps)) {
        return -1.0f;
    }
    if (R->criterion == 2u) {
        const REAL mag = F(vorticity_mag)(g, s, c, i);
        if (mag < 0.0f) {
            return -1.0f;
        }
        return mag > R->vort_split ? mag : -1.0f;
    }
    if (R->criterion == 3u) {
        /* within 2h of a domain face the clamp, not the air, truncates the support: no split there */
        REAL md[3];
        F(min_surface_distance)(P, p, md);
        if (!g->periodic && F(compmin3)(md) < h + h) {
            return -1.0f;
        }
        const REAL d = F(neighbour_deficit)(g, P, s, c, i);
        return d >= R->fs_split ? d : (REAL)-1;
    }
    const REAL* v = s->vel + 4 * (size_t)i;
    const REAL sp = SQRT(FMA(v[2], v[2], FMA(v[1], v[1], v[0] * v[0])));
    if (sp < R->vel_split) {
        return -1.0f;
    }
    return sp;
}

/* identifyMergeCandidates (cuda/src/algorithm/AdaptiveAlgorithm.cu:159-206): nearest neighbour with
 * r^2 < min(h_i,h_j)^2 and m_j < maxMass within the cells of [x - h_i, x + h_i]. Exact r^2 ties go to the
 * smaller id (the reference keeps the first one its loop meets). */
static uint32_t F(merge_candidate)(const orc_grid* g, const STATE* s, const orc_cells* c, uint32_t e,
                                REAL maxMass)
{
    const REAL* pe = s->pos + 4 * (size_t)e;
    const REAL he = s->h[e];
    REAL best = 3.402823466e38f;
    uint32_t bj = ORC_NONE;
    orc_iter it;
    uint32_t jb, je;
    float sh[3];
    float pef[4];
    it_init(&it, g, c->start, c->end, c->ex, ITPOS(pe, pef), (float)he);
    while (it_next(&it, &jb, &je, sh)) {
        for (uint32_t j = jb; j < je; j++) {
            if (j == e) {
                continue;
            }
            const REAL* pj = s->pos + 4 * (size_t)j;
            const REAL dx = pj[0] - pe[0], dy = pj[1] - pe[1], dz = pj[2] - pe[2];
            const REAL r2 = FMA(dz, dz, FMA(dy, dy, dx * dx));
            const REAL hj = s->h[j];
            const REAL hm = hj < he ? hj : he;
            if (r2 < hm * hm && s->m[j] < maxMass) {
                if (r2 < best || (r2 == best && s->id[j] < s->id[bj])) {
                    best = r2;
                    bj = j;
                }
            }
        }
    }
    return bj;
}


/* icosahedronVertices (cuda/src/algorithm/AdaptiveAlgorithm.cu:35-48), same order */
static void F(icosahedron)(REAL v[12][3])
{
    const REAL A = (REAL)ORC_PHI_F * (REAL)ORC_INVNORM_F, B = (REAL)ORC_INVNORM_F;
    const REAL t[12][3] = {{0.0f, A, B},  {0.0f, A, -B},  {0.0f, -A, -B}, {0.0f, -A, B},
                            {B, 0.0f, A},  {-B, 0.0f, A},  {B, 0.0f, -A},  {-B, 0.0f, -A},
                            {A, B, 0.0f},  {A, -B, 0.0f},  {-A, B, 0.0f},  {-A, -B, 0.0f}};
    memcpy(v, t, sizeof(t));
}

/* performMerges + calculateMergedSmoothingLength (cuda/src/algorithm/AdaptiveAlgorithm.cu:50-67, 236-275) */
static void F(merge_pair)(const orc_params* P, STATE* s, uint32_t i, uint32_t c)
{
    const REAL m1 = s->m[i], m2 = s->m[c];
    const REAL M = m1 + m2;
    REAL np[3], nv[3], na[3];
    for (int a = 0; a < 3; a++) {
        np[a] = FMA(m1, s->pos[4 * (size_t)i + a], m2 * s->pos[4 * (size_t)c + a]) / M;
        nv[a] = FMA(m1, s->vel[4 * (size_t)i + a], m2 * s->vel[4 * (size_t)c + a]) / M;
        na[a] = FMA(m1, s->acc[4 * (size_t)i + a], m2 * s->acc[4 * (size_t)c + a]) / M;
    }
    REAL d[2], W[2];
    const uint32_t idx[2] = {i, c};
    for (int k = 0; k < 2; k++) {
        const REAL* p = s->pos + 4 * (size_t)idx[k];
        const REAL dx = p[0] - np[0], dy = p[1] - np[1], dz = p[2] - np[2];
        d[k] = SQRT(FMA(dz, dz, FMA(dy, dy, dx * dx)));
        REAL invh, wc, dwc;
        F(kernel_consts)(s->h[idx[k]], &invh, &wc, &dwc);
        W[k] = F(kernel_w)(d[k], invh, wc);
    }
    const REAL denom = FMA(m1, W[0], m2 * W[1]);
    const REAL coef = ((REAL)16 * PI_R) / (REAL)21;
    const REAL hn = CBRT((coef * M) / denom);
    const REAL rn = P->r0 * CBRT(M / P->m0);
    for (int a = 0; a < 3; a++) {
        s->pos[4 * (size_t)i + a] = np[a];
        s->vel[4 * (size_t)i + a] = nv[a];
        s->acc[4 * (size_t)i + a] = na[a];
    }
    s->pos[4 * (size_t)i + 3] = 0.0f;
    s->vel[4 * (size_t)i + 3] = 0.0f;
    s->acc[4 * (size_t)i + 3] = 0.0f;
    s->m[i] = M;
    s->rad[i] = rn;
    s->h[i] = hn;
    s->rho[i] = 0.0f;
}

/* splitParticles (cuda/src/algorithm/AdaptiveAlgorithm.cu:69-117) with daughters at base .. base+11 */
static void F(split_one)(const orc_refine* R, STATE* s, uint32_t p, uint32_t base, uint32_t base_id)
{
    REAL ico[12][3];
    F(icosahedron)(ico);
    const REAL m = s->m[p], r = s->rad[p], h = s->h[p];
    const REAL dm = m * R->vertex_ratio, cm = m * R->center_ratio;
    const REAL nr = r * CBRT(dm / m);
    const REAL nh = R->alpha * h;
    REAL x[4], v[4], a[4];
    memcpy(x, s->pos + 4 * (size_t)p, sizeof(x));
    memcpy(v, s->vel + 4 * (size_t)p, sizeof(v));
    memcpy(a, s->acc + 4 * (size_t)p, sizeof(a));
    s->m[p] = cm;
    s->rad[p] = r * CBRT(cm / m);
    s->h[p] = nh;
    for (uint32_t k = 0; k < 12; k++) {
        const size_t q = base + k;
        for (int c = 0; c < 3; c++) {
            s->pos[4 * q + c] = x[c] + (ico[k][c] * R->eps) * h;
        }
        s->pos[4 * q + 3] = x[3];
        memcpy(s->vel + 4 * q, v, sizeof(v));
        memcpy(s->acc + 4 * q, a, sizeof(a));
        s->m[q] = dm;
        s->rad[q] = nr;
        s->h[q] = nh;
        s->rho[q] = 0.0f;
        s->id[q] = base_id + k;
    }
}

/* One refinement pass: performAdaptiveRefinement (cuda/src/simulation/AdaptiveSphSimulation.cu:102-113) with
 * identifyAndMergeParticles (:195-252) then, if particles were removed, identifyAndSplitParticles (:135-193).
 * Selection follows findTopParticlesToMerge/ToSplit (AdaptiveAlgorithm.cuh:56-131): stable sort of
 * (score, array slot) ascending for merge, descending for split; k = min(#score > 0, round(N*maxBatchRatio)).
 * Merge: non-eligible particles keep the reset candidate value 0, i.e. the particle in slot 0; pairs are
 * mutual candidates, the lower slot keeps. Split: the device count k bounds the kernel while the launch covers
 * ceil(budget/threadsPerBlock) blocks, budget = min(k, removed/12). Daughters are appended in split order. */
void F(refine_impl)(const orc_grid* g, const orc_params* P, const orc_refine* R, STATE* s, orc_cells* c,
                  orc_report* rep)
{
    orc_report local;
    if (rep == NULL) {
        memset(&local, 0, sizeof(local));
        rep = &local;
    }
    const uint32_t n = s->n;
    rep->frame = s->frame;
    rep->count_before = n;
    rep->merge_eligible = rep->merge_pairs = rep->removed = 0;
    rep->split_candidates = rep->split_budget = rep->splits = 0;
    rep->capacity_hit = 0;
    rep->count_after = n;
    if (n <= 1) {
        return;
    }
    const REAL minMass = R->min_mass_ratio * P->m0;
    const REAL maxMass = R->max_mass_ratio * P->m0;
    REAL* score = (REAL*)malloc(sizeof(REAL) * n);
    uint32_t* cand = (uint32_t*)malloc(sizeof(uint32_t) * n);
    uint8_t* flag = (uint8_t*)calloc(n, 1);

    uint32_t cpos = 0;
    for (uint32_t i = 0; i < n; i++) {
        score[i] = F(merge_score)(g, P, R, s, c, i, maxMass);
        cpos += score[i] > 0.0f;
    }
    const uint32_t lim = (uint32_t)roundf((float)n * R->max_batch_ratio);
    const uint32_t k = cpos < lim ? cpos : lim;
    rep->merge_eligible = k;
    uint32_t pairs = 0;
    if (k > 0) {
        /* (score, slot) ascending; ids are unique, so (sortable score, id) is a total order */
        uint32_t* sel = (uint32_t*)malloc(sizeof(uint32_t) * n);
        {
            orc_sel* tmp = (orc_sel*)malloc(sizeof(orc_sel) * n);
            for (uint32_t i = 0; i < n; i++) {
                tmp[i].key = SORTABLE(score[i]);
                tmp[i].id = s->id[i];
                tmp[i].slot = i;
            }
            qsort(tmp, n, sizeof(orc_sel), cmp_sel);
            for (uint32_t i = 0; i < n; i++) {
                sel[i] = tmp[i].slot;
            }
            free(tmp);
        }
        uint32_t slot0 = 0;
        for (uint32_t i = 1; i < n; i++) {
            if (s->id[i] < s->id[slot0]) {
                slot0 = i;
            }
        }
        for (uint32_t i = 0; i < n; i++) {
            cand[i] = slot0;
        }
        for (uint32_t q = 0; q < k; q++) {
            const uint32_t e = sel[q];
            cand[e] = F(merge_candidate)(g, s, c, e, maxMass);
        }
        free(sel);
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t cc = cand[i];
            if (cc == ORC_NONE) {
                continue;
            }
            if (cand[cc] == i && s->id[i] < s->id[cc]) {
                if (rep->keep_ids) {
                    rep->keep_ids[pairs] = s->id[i];
                }
                if (rep->removed_ids) {
                    rep->removed_ids[pairs] = s->id[cc];
                }
                F(merge_pair)(P, s, i, cc);
                flag[cc] = 1;
                pairs++;
            }
        }
    }
    rep->merge_pairs = pairs;
    if (pairs > 0) {
        /* stable compaction (compactParticles, AdaptiveAlgorithm.cu:130-157, done out of place) */
        uint32_t w = 0;
        for (uint32_t i = 0; i < n; i++) {
            if (flag[i]) {
                continue;
            }
            if (w != i) {
                memcpy(s->pos + 4 * (size_t)w, s->pos + 4 * (size_t)i, sizeof(SREAL) * 4);
                memcpy(s->vel + 4 * (size_t)w, s->vel + 4 * (size_t)i, sizeof(SREAL) * 4);
                memcpy(s->acc + 4 * (size_t)w, s->acc + 4 * (size_t)i, sizeof(SREAL) * 4);
                s->rho[w] = s->rho[i];
                s->rad[w] = s->rad[i];
                s->h[w] = s->h[i];
                s->m[w] = s->m[i];
                s->id[w] = s->id[i];
                c->keys[w] = c->keys[i];
            }
            w++;
        }
        const uint32_t removed = n - w;
        rep->removed = removed;
        s->n = w;
        const uint32_t n2 = w;
        if (R->criterion == 2u || R->criterion == 3u) { /* criteria that walk neighbours: cells of the compacted set */
            orc_cells_from_keys(g, n2, c->keys, c->start, c->end);
        }
        uint32_t cs = 0;
        for (uint32_t i = 0; i < n2; i++) {
            score[i] = F(split_score)(g, P, R, s, c, i, minMass);
            cs += score[i] > 0.0f;
        }
        const uint32_t lim2 = (uint32_t)roundf((float)n2 * R->max_batch_ratio);
        const uint32_t ks = cs < lim2 ? cs : lim2;
        rep->split_candidates = ks;
        const uint32_t budget = ks < removed / 12u ? ks : removed / 12u;
        rep->split_budget = budget;
        if (budget > 0) {
            const uint32_t tpb = P->threads_per_block ? P->threads_per_block : 256u;
            uint64_t launched = (uint64_t)((budget + tpb - 1) / tpb) * tpb;
            const uint32_t M = (uint64_t)ks < launched ? ks : (uint32_t)launched;
            orc_sel* tmp = (orc_sel*)malloc(sizeof(orc_sel) * n2);
            for (uint32_t i = 0; i < n2; i++) {
                tmp[i].key = SORTABLE_DESC(score[i]);
                tmp[i].id = s->id[i];
                tmp[i].slot = i;
            }
            qsort(tmp, n2, sizeof(orc_sel), cmp_sel);
            uint32_t done = 0;
            for (uint32_t r = 0; r < M; r++) {
                const uint64_t end = (uint64_t)n2 + 12ull * (r + 1);
                if (end > s->cap) {
                    rep->capacity_hit = 1;
                    break;
                }
                const uint32_t p = tmp[r].slot;
                if (rep->split_ids) {
                    rep->split_ids[r] = s->id[p];
                }
                F(split_one)(R, s, p, n2 + 12u * r, s->next_id + 12u * r);
                done++;
            }
            free(tmp);
            rep->splits = done;
            s->n = n2 + 12u * done;
            s->next_id += 12u * done;
        }
    }
    rep->count_after = s->n;
    free(score);
    free(cand);
    free(flag);
}

