/*
 * ekg_oracle.c -- FP64 CPU restatement of the EkgSim simulation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU engine: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it.  The engine in
 * ekgsim_gb300/ never links, loads or calls it.
 *
 * Every function follows the reference operation for operation (same evaluation order,
 * same rounding points), compiled with -ffp-contract=off so that no multiply-add is fused:
 *   - activation times (cellular automaton, Dijkstra): simlib/simulator.cpp:212-286
 *   - Wohlfart AP:                                      simlib/Wohlfart.h:195-203
 *   - cell AP with k8 -= at:                            simlib/simulator.cpp:154-170
 *   - ECG run (bordered raster walk, dipoles, leads):   simlib/simulator.cpp:452-550
 *   - apIndex de-duplication (first-seen raster order): simlib/simulator.cpp:561-621
 *   - genes -> layer APs, interpolation, violation:     sim.cpp:751-916, :582-596, :705-709
 *   - steepest descent:                                 nonlinearFit.h:92-168
 *   - interpolation evaluator / apd90:                  sim.cpp:91-313, simlib/Wohlfart.h:206-223
 *   - lead u/v basis and displacement:                  simlib/sim_lib.h:167-208
 *   - criteria (pearson, rms, vector corr, devFromLinear): vectorMath.h:180-404, sim.cpp:600-702
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define EKGO_OK 0
#define EKGO_ERR_NO_START -1
#define EKGO_ERR_TRANSFER -2
#define EKGO_ERR_ARG -3
#define EKGO_ERR_NOMEM -4

/* ------------------------------------------------------------------ Wohlfart AP */
/* WohlfartPlus::operator[] (simlib/Wohlfart.h:195-203), same operand order. */
static double wohl(const double *k, double t) {
    return (1.0 / (1.0 + exp(-k[1] * t)))
         * (k[2] * ((1.0 - k[3]) * exp(-k[4] * t) + k[3]))
         * (exp(-k[5] * t) * (1 - pow((1 + exp(-k[7] * (t - k[8])
              + log(pow(2, (k[7] / k[6])) - 1))), -(k[6] / k[7]))))
         + k[0];
}

double ekgo_wohl(const double *k, double t) { return wohl(k, t); }

/* An ActionPotential: 9 k values (k8 already shifted by -at) plus at (simlib/simulator.h:468-480). */
typedef struct { double k[9]; double at; } ap_t;

static void ap_init(ap_t *ap, const double *k, double at) {   /* simlib/simulator.cpp:154-165 */
    memcpy(ap->k, k, 9 * sizeof(double));
    ap->k[8] -= at;
    ap->at = at;
}
static double ap_eval(const ap_t *ap, double t) { return wohl(ap->k, t - ap->at); }  /* :168-170 */

/* ------------------------------------------------------------- activation times */
typedef struct { double t; int64_t idx; } pq_el;

static void pq_push(pq_el *h, int64_t *n, double t, int64_t idx) {
    int64_t i = (*n)++;
    while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (h[p].t <= t) break;
        h[i] = h[p];
        i = p;
    }
    h[i].t = t; h[i].idx = idx;
}
static pq_el pq_pop(pq_el *h, int64_t *n) {
    pq_el top = h[0], last = h[--(*n)];
    int64_t i = 0;
    for (;;) {
        int64_t c = 2 * i + 1;
        if (c >= *n) break;
        if (c + 1 < *n && h[c + 1].t < h[c].t) c++;
        if (h[c].t >= last.t) break;
        h[i] = h[c];
        i = c;
    }
    h[i] = last;
    return top;
}

/*
 * Simulation::calculateExcitationSequence + exciteElement (simlib/simulator.cpp:212-286).
 * raw[z][y][x] holds the file's layer values: 0 empty, >0 layer, <0 stimulus voxel of layer
 * |v| (simlib/matrix.h:125-129).  Output at[] (0 = empty or unreachable) and the stripped layer.
 * The 26-neighbour cube is used for 3D grids; for nz == 1 the in-plane 8-neighbourhood of the
 * reference is the same set restricted to the grid.
 * lag = T[L(src)][L(dst)] * sqrt(|d|^2); time(dst) = time(src) + lag, popped in time order.
 */
int ekgo_activation(int nz, int ny, int nx, const int32_t *raw, int ntm, const double *tm,
                    double *at, int32_t *layer) {
    int64_t n = (int64_t)nz * ny * nx;
    int64_t cap = 27 * n + 16, hn = 0;
    pq_el *heap = (pq_el *)malloc((size_t)cap * sizeof(pq_el));
    if (!heap) return EKGO_ERR_NOMEM;
    int64_t nstart = 0;
    for (int64_t i = 0; i < n; ++i) {
        at[i] = 0.0;
        int32_t v = raw[i];
        if (v < 0) { layer[i] = -v; pq_push(heap, &hn, 1.0, i); ++nstart; }
        else layer[i] = v;
    }
    if (nstart == 0) { free(heap); return EKGO_ERR_NO_START; }
    while (hn > 0) {
        pq_el a = pq_pop(heap, &hn);
        if (at[a.idx] != 0) continue;
        at[a.idx] = a.t;
        int64_t z = a.idx / ((int64_t)ny * nx), y = (a.idx / nx) % ny, x = a.idx % nx;
        int32_t ls = layer[a.idx];
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    if (!dz && !dy && !dx) continue;
                    int64_t z2 = z - dz, y2 = y - dy, x2 = x - dx;
                    if (z2 < 0 || z2 >= nz || y2 < 0 || y2 >= ny || x2 < 0 || x2 >= nx) continue;
                    int64_t j = (z2 * ny + y2) * nx + x2;
                    if (layer[j] <= 0 || at[j] != 0) continue;
                    if (ls >= ntm || layer[j] >= ntm) { free(heap); return EKGO_ERR_TRANSFER; }
                    double lag = tm[(int64_t)ls * ntm + layer[j]];
                    lag *= sqrt((double)(dz * dz + dy * dy + dx * dx));
                    if (hn >= cap) { free(heap); return EKGO_ERR_NOMEM; }
                    pq_push(heap, &hn, a.t + lag, j);
                }
    }
    free(heap);
    return EKGO_OK;
}

/* ------------------------------------------------------------ neighbourhoods */
/* Neighbourhood::create with the callbacks of simlib/simulator.h:334-384, in creation order
 * (active[0], active[1], active[2] each 0..2; dif = active - (1,1,1)).
 * code 0 = "3D4" (callback3x2N: 8 body diagonals), 1 = "3D8"/"cube" (26), 2 = "2D4"
 * (callback4N), 3 = "2D8" (callback8N).  Returns the count; dif is [n][3] in (z,y,x). */
int ekgo_neighbourhood(int code, int *dif) {
    int cnt = 0;
    for (int a0 = 0; a0 < 3; ++a0)
        for (int a1 = 0; a1 < 3; ++a1)
            for (int a2 = 0; a2 < 3; ++a2) {
                int d0 = abs(a0 - 1), d1 = abs(a1 - 1), d2 = abs(a2 - 1);
                int ok = 0;
                if (code == 0) {
                    int mn = d0 < d1 ? d0 : d1; mn = mn < d2 ? mn : d2;
                    int mx = d0 > d1 ? d0 : d1; mx = mx > d2 ? mx : d2;
                    ok = (mn == 1 && mx == 1);
                } else if (code == 1) {
                    int mx = d0 > d1 ? d0 : d1; mx = mx > d2 ? mx : d2;
                    ok = (mx == 1);
                } else if (code == 2) {
                    int mn = d1 < d2 ? d1 : d2, mx = d1 > d2 ? d1 : d2;
                    ok = (mn == 1 && mx == 1 && d0 == 0);
                } else if (code == 3) {
                    int mx = d1 > d2 ? d1 : d2;
                    ok = (mx == 1 && d0 == 0);
                }
                if (ok) {
                    dif[3 * cnt + 0] = a0 - 1; dif[3 * cnt + 1] = a1 - 1; dif[3 * cnt + 2] = a2 - 1;
                    ++cnt;
                }
            }
    return cnt;
}

/* ------------------------------------------------------------ apIndex de-duplication */
typedef struct { int32_t layer; double at; int64_t first; } key_t_;
static int key_cmp(const void *a, const void *b) {
    const key_t_ *x = (const key_t_ *)a, *y = (const key_t_ *)b;
    if (x->layer != y->layer) return x->layer < y->layer ? -1 : 1;
    if (x->at != y->at) return x->at < y->at ? -1 : 1;
    return (x->first < y->first) ? -1 : (x->first > y->first);
}

/* Simulation::setApIndices (simlib/simulator.cpp:561-621): apIndex = order of first appearance
 * of each (layer, at) pair in raster order.  Writes ap_index[] for every non-empty voxel
 * (-1 for empty) and the (layer, at) of each index; returns the number of unique pairs. */
int64_t ekgo_ap_indices(int64_t n, const int32_t *layer, const double *at, int64_t *ap_index,
                        int32_t *ap_layer, double *ap_at) {
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) if (layer[i] > 0) ++m;
    key_t_ *keys = (key_t_ *)malloc((size_t)(m ? m : 1) * sizeof(key_t_));
    if (!keys) return EKGO_ERR_NOMEM;
    int64_t j = 0;
    for (int64_t i = 0; i < n; ++i) {
        ap_index[i] = -1;
        if (layer[i] > 0) { keys[j].layer = layer[i]; keys[j].at = at[i]; keys[j].first = i; ++j; }
    }
    qsort(keys, (size_t)m, sizeof(key_t_), key_cmp);
    /* groups are contiguous; the group's first element has the smallest raster index */
    int64_t ng = 0;
    int64_t *gfirst = (int64_t *)malloc((size_t)(m ? m : 1) * sizeof(int64_t));
    for (int64_t a = 0; a < m; ) {
        int64_t b = a;
        while (b < m && keys[b].layer == keys[a].layer && keys[b].at == keys[a].at) ++b;
        gfirst[ng++] = keys[a].first;
        for (int64_t c = a; c < b; ++c) ap_index[keys[c].first] = -2 - (ng - 1); /* temp: group id */
        a = b;
    }
    /* number the groups by first appearance: walk raster order */
    int64_t *gid2ap = (int64_t *)malloc((size_t)(ng ? ng : 1) * sizeof(int64_t));
    for (int64_t g = 0; g < ng; ++g) gid2ap[g] = -1;
    int64_t next = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (layer[i] <= 0) continue;
        int64_t g = -2 - ap_index[i];
        if (gid2ap[g] < 0) {
            gid2ap[g] = next;
            if (ap_layer) ap_layer[next] = layer[i];
            if (ap_at) ap_at[next] = at[i];
            ++next;
        }
        ap_index[i] = gid2ap[g];
    }
    free(gid2ap); free(gfirst); free(keys);
    return ng;
}

/* ------------------------------------------------------------------- ECG run */
/*
 * Simulation::run (simlib/simulator.cpp:452-550) in the reference's summation order:
 *   for each non-empty voxel x in raster order (bordered index = original + 1):
 *     cell[i] = AP_x(t_i); dipole[i] = 0
 *     for each neighbour d in creation order with L(x - d) > 0: dipole[i] += d * (AP_{x-d}(t_i) - cell[i])
 *     for each lead: m = r - x; m *= 1/(|m|^2 * sqrt(|m|^2)); ecg[l][i] += ((0 + m0 D0) + m1 D1) + m2 D2
 * AP values come from a per-(layer, at) table, which is bit-identical to evaluating each
 * voxel's AP in place (same function, same arguments).  Time t_i is accumulated by += dt
 * from start, as in the reference.  Work is split over threads by time step, so every ecg[l][i]
 * sum still runs over the voxels in raster order.
 * layer_k: nlayers x 9 layer AP coefficients (layer 1 at row 0); lead_zyx: nlead x 3 (z,y,x).
 */
int ekgo_run(int nz, int ny, int nx, const int32_t *layer, const double *at,
             int nlayers, const double *layer_k, int nlead, const double *lead_zyx,
             int nhood_code, double start, double length, double dt, double *ecg, int nthreads) {
    int64_t n = (int64_t)nz * ny * nx;
    int64_t steps = (int64_t)ceil(length / dt);
    if (steps <= 0 || nlead < 0) return EKGO_ERR_ARG;
    /* the neighbour loop of the reference runs while simTime < start + length */
    {
        int64_t cnt = 0;
        double total = length + start;
        for (double s = start; s < total; s += dt) ++cnt;
        if (cnt != steps) return EKGO_ERR_ARG;
    }
    double *tt = (double *)malloc((size_t)steps * sizeof(double));
    { double s = start; for (int64_t i = 0; i < steps; ++i) { tt[i] = s; s += dt; } }

    int64_t *api = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int32_t *apl = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    double *apat = (double *)malloc((size_t)n * sizeof(double));
    int64_t na = ekgo_ap_indices(n, layer, at, api, apl, apat);
    if (na < 0) return (int)na;
    for (int64_t a = 0; a < na; ++a)
        if (apl[a] < 1 || apl[a] > nlayers) { free(tt); free(api); free(apl); free(apat); return EKGO_ERR_ARG; }
    ap_t *aps = (ap_t *)malloc((size_t)(na ? na : 1) * sizeof(ap_t));
    for (int64_t a = 0; a < na; ++a) ap_init(&aps[a], layer_k + 9 * (apl[a] - 1), apat[a]);

    int dif[26 * 3];
    int nnb = ekgo_neighbourhood(nhood_code, dif);

    /* compact list of non-empty voxels in raster order with their neighbours and lead vectors */
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) if (layer[i] > 0) ++m;
    int64_t *vap = (int64_t *)malloc((size_t)(m ? m : 1) * sizeof(int64_t));
    int64_t *nb = (int64_t *)malloc((size_t)(m ? m : 1) * nnb * sizeof(int64_t));
    double *mv = (double *)malloc((size_t)(m ? m : 1) * (nlead ? nlead : 1) * 3 * sizeof(double));
    int64_t v = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (layer[i] <= 0) continue;
        int64_t z = i / ((int64_t)ny * nx), y = (i / nx) % ny, x = i % nx;
        vap[v] = api[i];
        for (int q = 0; q < nnb; ++q) {
            int64_t z2 = z - dif[3 * q], y2 = y - dif[3 * q + 1], x2 = x - dif[3 * q + 2];
            int64_t j = -1;
            if (z2 >= 0 && z2 < nz && y2 >= 0 && y2 < ny && x2 >= 0 && x2 < nx) {
                int64_t jj = (z2 * ny + y2) * nx + x2;
                if (layer[jj] > 0) j = api[jj];
            }
            nb[v * nnb + q] = j;
        }
        for (int l = 0; l < nlead; ++l) {
            double m0 = lead_zyx[3 * l + 0] - (double)(z + 1);
            double m1 = lead_zyx[3 * l + 1] - (double)(y + 1);
            double m2 = lead_zyx[3 * l + 2] - (double)(x + 1);
            double s = m0 * m0; s += m1 * m1; s += m2 * m2;
            double f = 1.0 / (s * sqrt(s));
            m0 *= f; m1 *= f; m2 *= f;
            mv[(v * nlead + l) * 3 + 0] = m0;
            mv[(v * nlead + l) * 3 + 1] = m1;
            mv[(v * nlead + l) * 3 + 2] = m2;
        }
        ++v;
    }
    for (int64_t i = 0; i < (int64_t)nlead * steps; ++i) ecg[i] = 0.0;

    const int64_t B = 64;   /* time steps per block */
    double *tab = (double *)malloc((size_t)(na ? na : 1) * B * sizeof(double));
    if (!tab) return EKGO_ERR_NOMEM;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    for (int64_t b0 = 0; b0 < steps; b0 += B) {
        int64_t nb_ = steps - b0 < B ? steps - b0 : B;
#pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < na; ++a)
            for (int64_t j = 0; j < nb_; ++j) tab[a * B + j] = ap_eval(&aps[a], tt[b0 + j]);
        /* each task owns J consecutive steps; per (lead, step) the sum still runs in raster order */
        enum { J = 8 };
#pragma omp parallel for schedule(dynamic, 1)
        for (int64_t j0 = 0; j0 < nb_; j0 += J) {
            int64_t nj = nb_ - j0 < J ? nb_ - j0 : J;
            double *acc = (double *)malloc((size_t)(nlead ? nlead : 1) * J * sizeof(double));
            for (int64_t q = 0; q < (int64_t)nlead * J; ++q) acc[q] = 0.0;
            for (int64_t u = 0; u < m; ++u) {
                const double *cell = tab + vap[u] * B + j0;
                double D0[J], D1[J], D2[J];
                for (int64_t j = 0; j < nj; ++j) { D0[j] = 0.0; D1[j] = 0.0; D2[j] = 0.0; }
                for (int q = 0; q < nnb; ++q) {
                    int64_t k = nb[u * nnb + q];
                    if (k < 0) continue;
                    const double *nv = tab + k * B + j0;
                    double f0 = (double)dif[3 * q + 0], f1 = (double)dif[3 * q + 1], f2 = (double)dif[3 * q + 2];
                    for (int64_t j = 0; j < nj; ++j) {
                        double vd = nv[j] - cell[j];
                        D0[j] += f0 * vd;
                        D1[j] += f1 * vd;
                        D2[j] += f2 * vd;
                    }
                }
                for (int l = 0; l < nlead; ++l) {
                    const double *mm = mv + (u * nlead + l) * 3;
                    double *al = acc + (int64_t)l * J;
                    for (int64_t j = 0; j < nj; ++j) {
                        double r = 0.0;
                        r += mm[0] * D0[j]; r += mm[1] * D1[j]; r += mm[2] * D2[j];
                        al[j] += r;
                    }
                }
            }
            for (int l = 0; l < nlead; ++l)
                for (int64_t j = 0; j < nj; ++j) ecg[l * steps + b0 + j0 + j] = acc[(int64_t)l * J + j];
            free(acc);
        }
    }
    free(tab); free(mv); free(nb); free(vap); free(aps); free(apat); free(apl); free(api); free(tt);
    return EKGO_OK;
}

/* -------------------------------------------------- gene -> layer AP construction */
static double der(double x, const ap_t *ap) { return 100 * (ap_eval(ap, x + 0.01) - ap_eval(ap, x)); }  /* sim.cpp:75-78 */

/* WohlfartPlus::apd90 (simlib/Wohlfart.h:206-223) */
static double apd90(const double *k) {
    double d[1000];
    for (int di = 0; di < 1000; ++di) d[di] = wohl(k, (double)di);
    double target = k[0] + k[2] * 0.1;
    double time = -1.0;
    for (int di = 1; di < 1000; ++di)
        if ((d[di - 1] > target) && (d[di] <= target)) {
            double a = (double)(di - 1), wa = d[di - 1] - target, b = (double)di, wb = target - d[di];
            time = (a * wa + b * wb) / (wa + wb);
        }
    return time;
}

typedef struct { double k, n, x1, x2; } connector_t;
typedef struct { connector_t c[15]; int nc; double pts[30]; int np; int overrun; } evaluator_t;

/* WohlfartInterpolationEvaluator::distributeConnectors (sim.cpp:204-264).  The reference
 * reads ap1y[i1 + 1] without a bound check; 'overrun' records if that would step past 699. */
static void set_border_aps(evaluator_t *e, const ap_t *ap1, const ap_t *ap2) {
    const size_t numPoints = 15, startX = 10;
    double apd1 = apd90(ap1->k), apd2 = apd90(ap2->k);
    double len1 = 0.0, len2 = 0.0;
    static __thread double ap1y[701], ap2y[701];
    const double xs = 0.1;
    for (size_t i = 0; i < 700; ++i) { ap1y[i] = ap_eval(ap1, (double)i); ap2y[i] = ap_eval(ap2, (double)i); }
    ap1y[700] = ap1y[699]; ap2y[700] = ap2y[699];
    size_t e1 = (size_t)ceil(apd1), e2 = (size_t)ceil(apd2);
    if (apd1 < 0) e1 = 0;
    if (apd2 < 0) e2 = 0;
    size_t lim1 = e1 < 700 ? e1 : 700, lim2 = e2 < 700 ? e2 : 700;
    for (size_t i = startX + 1; i < lim1; ++i) { double q = ap1y[i] - ap1y[i - 1]; len1 += sqrt(q * q + xs); }
    for (size_t i = startX; i < lim2; ++i) { double q = ap2y[i] - ap2y[i - 1]; len2 += sqrt(q * q + xs); }
    double cur1 = 0.0, cur2 = 0.0;
    size_t i1 = startX, i2 = startX;
    e->nc = 0; e->overrun = 0;
    connector_t lc; lc.k = 100;
    for (size_t i = 0; i < numPoints; ++i) {
        double targetLen = (double)i * len1 / (double)(numPoints - 2);
        for (double l1 = cur1; (l1 < targetLen) && (i1 < 700); ++i1) {
            if (i1 + 1 >= 700) e->overrun = 1;
            double q = ap1y[i1 + 1] - ap1y[i1]; l1 += sqrt(q * q + xs);
        }
        cur1 = targetLen;
        targetLen = (double)i * len2 / (double)(numPoints - 2);
        for (double l2 = cur2; (l2 < targetLen) && (i2 < 700); ++i2) {
            if (i2 + 1 >= 700) e->overrun = 1;
            double q = ap2y[i2 + 1] - ap2y[i2]; l2 += sqrt(q * q + xs);
        }
        cur2 = targetLen;
        if (i1 >= 700 || i2 >= 700) e->overrun = 1;
        lc.x1 = (double)i1;
        lc.x2 = (double)i2;
        if (i1 == i2) lc.x2 += 0.001;
        lc.k = (ap1y[i1] - ap2y[i2]) / (lc.x1 - lc.x2);
        lc.n = ap2y[i2] - lc.k * (double)i2;
        e->c[e->nc++] = lc;
    }
}

static void setup_ratio(evaluator_t *e, double ratio) {   /* sim.cpp:268-277 */
    e->np = 0;
    for (int i = 0; i < e->nc; ++i) {
        double x = e->c[i].x1 + (e->c[i].x2 - e->c[i].x1) * ratio;
        e->pts[e->np++] = x;
        e->pts[e->np++] = e->c[i].k * x + e->c[i].n;
    }
}

static double eval_fit(const evaluator_t *e, const ap_t *ap) {   /* sim.cpp:174-185 */
    double sum = 0;
    for (int i = 0; i < e->np; i += 2) { double q = ap_eval(ap, e->pts[i]) - e->pts[i + 1]; sum += q * q; }
    return sum;
}

/* steepestDescend (nonlinearFit.h:92-168) with Vec = ActionPotential (9 k values). */
static void steepest(const evaluator_t *e, ap_t *x0, const ap_t *d, double stepSize, double epsilon, int iterations) {
    ap_t grad = *x0, oldGrad = grad, move = *d;
    for (int i = 0; i < 9; ++i) oldGrad.k[i] = 0;
    double y0 = eval_fit(e, x0);
    for (; (iterations > 0) && (y0 > epsilon); --iterations) {
        int stepChange = 0;
        for (int i = 0; i < 9; ++i) {
            ap_t x1 = *x0;
            if (d->k[i] != 0) {
                x1.k[i] += d->k[i] * .001;
                grad.k[i] = (eval_fit(e, &x1) - y0) / (d->k[i] * .001);
                if (grad.k[i] * oldGrad.k[i] < 0) { move.k[i] *= 0.5; stepChange = 1; }
                else if (fabs(grad.k[i]) > 0.75 * fabs(oldGrad.k[i])) move.k[i] *= 1.5;
            } else {
                grad.k[i] = 0;
            }
        }
        oldGrad = grad;
        ap_t x1 = *x0;
        for (int i = 0; i < 9; ++i) x1.k[i] -= stepSize * ((grad.k[i] > 0) ? move.k[i] : -move.k[i]);
        double y1 = eval_fit(e, &x1);
        if (y1 < y0) { y0 = y1; *x0 = x1; }
        else if (!stepChange) stepSize *= 0.5;
    }
}

static void combine(ap_t *dest, const ap_t *s1, const ap_t *s2, double ratio) {   /* sim.cpp:705-709 */
    for (int i = 0; i < 9; ++i) dest->k[i] = s1->k[i] * (1 - ratio) + s2->k[i] * ratio;
}

static double violation_of(const double *k, int i, const double *kmin, const double *kmax) {   /* sim.cpp:582-589 */
    if (k[i] < kmin[i]) return kmin[i] - k[i];
    if (k[i] > kmax[i]) return k[i] - kmax[i];
    return 0;
}

/*
 * SimImplementation::simUsingBorderAps / simUsingBorderAndMidAps (sim.cpp:751-916).
 * interp: 1 = endo-epi, 2 = endo-mid-epi.  base: nbase x 9 (front = row 0, back = last row).
 * free_mask: bit i set when k_i is a free gene.  genes: the Wohlfart genes only.
 * Writes nlayers x 9 layer APs and the violation.  Returns 0, or 1 when the connector walk
 * of the interpolation evaluator would read past the reference's 700-sample buffer.
 */
int ekgo_layer_aps(int nlayers, int nbase, const double *base, const double *kmin, const double *kmax,
                   unsigned free_mask, int interp, double mid_position, const double *genes,
                   double *out_k, double *violation) {
    ap_t *aps = (ap_t *)calloc((size_t)nlayers, sizeof(ap_t));
    ap_t temp;
    int gi = 0, overrun = 0;
    double viol = 0.0;
    static const double kd[9] = {0, 0, 0, 0.001, 0, 0.00005, 0.0005, 0.01, 0.2};
    ap_t d; ap_init(&d, kd, 0);
    const double *front = base, *back = base + 9 * (nbase - 1);
    evaluator_t ev;
#define FILL_GENES(src) do { ap_init(&temp, (src), 0); \
        for (int i = 0; i < 9; ++i) if (free_mask & (1u << i)) { temp.k[i] = genes[gi++]; viol += violation_of(temp.k, i, kmin, kmax); } } while (0)
    if (interp == 1) {
        FILL_GENES(front); ap_init(&aps[0], temp.k, 0);
        FILL_GENES(back);  ap_init(&aps[nlayers - 1], temp.k, 0);
        set_border_aps(&ev, &aps[0], &aps[nlayers - 1]); overrun |= ev.overrun;
        for (int i = 1; i < nlayers - 1; ++i) {
            double ratio = i / (double)(nlayers - 1);
            setup_ratio(&ev, ratio);
            aps[i] = aps[i - 1];
            combine(&aps[i], &aps[0], &aps[nlayers - 1], ratio);
            steepest(&ev, &aps[i], &d, 0.5, 1e-3, 100);
        }
    } else {
        size_t mid = (size_t)floor(mid_position * (nlayers - 1) + 0.5);
        FILL_GENES(front); ap_init(&aps[0], temp.k, 0);
        FILL_GENES(back);  ap_init(&aps[mid], temp.k, 0);
        FILL_GENES(back);  ap_init(&aps[nlayers - 1], temp.k, 0);
        set_border_aps(&ev, &aps[0], &aps[nlayers - 1]); overrun |= ev.overrun;
        for (size_t i = 1; i + 1 < (size_t)nlayers; ++i) {
            if (i < mid) {
                double ratio = i / (double)mid;
                set_border_aps(&ev, &aps[0], &aps[mid]); overrun |= ev.overrun;
                setup_ratio(&ev, ratio);
                aps[i] = aps[i - 1];
                combine(&aps[i], &aps[0], &aps[mid], ratio);
            } else if (i > mid) {
                double ratio = (i - mid) / (double)(nlayers - mid - 1);
                if ((i - mid) == 1) { set_border_aps(&ev, &aps[mid], &aps[nlayers - 1]); overrun |= ev.overrun; }
                setup_ratio(&ev, ratio);
                aps[i] = aps[i - 1];
                combine(&aps[i], &aps[mid], &aps[nlayers - 1], ratio);
            }
            if (i != mid) steepest(&ev, &aps[i], &d, 0.5, 1e-3, 100);
        }
    }
#undef FILL_GENES
    for (int i = 0; i < nlayers; ++i) memcpy(out_k + 9 * i, aps[i].k, 9 * sizeof(double));
    *violation = viol;
    free(aps);
    return overrun;
}

/* ------------------------------------------------------------- lead movement */
/* EkgSim::loadMeasuringPoints u/v basis and moveMeasuringPoints (simlib/sim_lib.h:167-208),
 * coordinates in (z,y,x) order: x = (0,0,1); u = -normalize(x cross p); v = normalize(u_raw cross p)
 * where u_raw is the un-negated cross product. */
static void normalize3(double *v) {
    double s = v[0] * v[0]; s += v[1] * v[1]; s += v[2] * v[2];
    double l = sqrt(s);
    if (l != 0) { double f = 1.0 / l; v[0] *= f; v[1] *= f; v[2] *= f; }
    else { v[0] *= 0.0; v[1] *= 0.0; v[2] *= 0.0; }
}
static void cross3(const double *a, const double *b, double *ab) {
    ab[0] = a[1] * b[2] - a[2] * b[1];
    ab[1] = a[2] * b[0] - a[0] * b[2];
    ab[2] = a[0] * b[1] - a[1] * b[0];
}
void ekgo_move_leads(int nlead, const double *orig_zyx, const double *disp, double *out_zyx) {
    for (int i = 0; i < nlead; ++i) {
        const double *p = orig_zyx + 3 * i;
        double x[3] = {0, 0, 1}, u[3], v[3];
        cross3(x, p, u);
        cross3(u, p, v);
        u[0] *= -1; u[1] *= -1; u[2] *= -1;
        normalize3(u); normalize3(v);
        double du = disp ? disp[2 * i] : 0.0, dv = disp ? disp[2 * i + 1] : 0.0;
        /* originalMeasuringPositions[i] + u_disp * vectorU[i] + v_disp * vectorV[i] */
        for (int c = 0; c < 3; ++c) {
            double su = du * u[c];
            double sv = dv * v[c];
            out_zyx[3 * i + c] = (p[c] + su) + sv;
        }
    }
}

/* ------------------------------------------------------------------- criteria */
static void mean_var(double *mean, double *var, const double *s, int64_t start, int64_t end) {   /* vectorMath.h:180-188 */
    double inv = 1.0 / (double)(end - start);
    double sum = 0;
    for (int64_t i = start; i < end; ++i) sum += s[i];
    *mean = sum * inv;
    double v = 0;
    for (int64_t i = start; i < end; ++i) { double q = s[i] - *mean; v += q * q; }
    *var = v * inv;
}

/* Comparison of one simulated lead a (na samples) against target b (nb), offset 0.
 * mode 1 rms, 2 1-pearson, 3 devFromLinear (with target offset bofs), 4 1-vector-correlation.
 * (vectorMath.h:287-404, sim.cpp:618-648). */
double ekgo_compare(int mode, const double *a, int64_t na, const double *b, int64_t nb, double bofs) {
    int64_t len = na < nb ? na : nb;
    if (mode == 2) {
        double ma, va, mb, vb;
        mean_var(&ma, &va, a, 0, len); va = sqrt(va);
        mean_var(&mb, &vb, b, 0, len); vb = sqrt(vb);
        double res = 0;
        for (int64_t i = 0; i < len; ++i) res += (a[i] - ma) * (b[i] - mb);
        double cov = res / (double)len;
        return 1.0 - cov / (va * vb);
    } else if (mode == 4) {
        double ab = 0, aa = 0, bb = 0;
        for (int64_t i = 0; i < len; ++i) ab += a[i] * b[i];
        for (int64_t i = 0; i < len; ++i) aa += a[i] * a[i];
        for (int64_t i = 0; i < len; ++i) bb += b[i] * b[i];
        return 1.0 - ab / (sqrt(aa) * sqrt(bb));
    } else if (mode == 1) {
        double *q = (double *)malloc((size_t)(len ? len : 1) * sizeof(double));
        for (int64_t i = 0; i < len; ++i) { double x = a[i] - b[i]; q[i] = x * x; }
        double mean, var;
        mean_var(&mean, &var, q, 0, len);
        free(q);
        return sqrt(mean);
    } else {
        double amin = a[0], amax = a[0];
        for (int64_t i = 1; i < na; ++i) { if (a[i] < amin) amin = a[i]; else if (a[i] > amax) amax = a[i]; }
        double amult = 1.0 / (amax - amin);
        double *q = (double *)malloc((size_t)(len ? len : 1) * sizeof(double));
        for (int64_t i = 0; i < len; ++i) q[i] = (a[i] * amult + bofs) / (b[i] + bofs);
        double mean, var;
        mean_var(&mean, &var, q, 0, len);
        free(q);
        if (var == 0) return 1 / 1e-30;
        return sqrt(var);
    }
}

/* Clamp of sim.cpp:676-681: negative, non-finite or non-normal -> 2e10. */
double ekgo_clamp(double c) {
    if ((c < 0) || !isfinite(c) || !isnormal(c)) return 2e10;
    return c;
}

/* ------------------------------------------------------ reference-cost CPU baseline */
/*
 * Simulation::run with the reference's own cost structure (simlib/simulator.cpp:452-550): every
 * cell AP and every neighbour AP is evaluated in place, once per step, exactly as the reference
 * does (about nine Wohlfart evaluations per voxel-step), single-threaded, including the apIndex
 * build (setApIndices, :561-621).  Used only to time the CPU baseline; results are bit-identical
 * to ekgo_run.  `steps_limit` > 0 runs only the first steps_limit steps (a bounded sample).
 */
/* Steps [k0, k1) of the reference's voxel-major loop (ecg is nlead x (k1 - k0)): the time of step k
 * is start advanced by += dt k times, as simTime is in simlib/simulator.cpp:496-500, 519, so any
 * split of the time axis into ranges gives the same values as one pass over all of it. */
int ekgo_run_naive_range(int nz, int ny, int nx, const int32_t *layer, const double *at, int nlayers,
                         const double *layer_k, int nlead, const double *lead_zyx, int nhood_code, double start,
                         double length, double dt, int64_t k0, int64_t k1, double *ecg) {
    int64_t n = (int64_t)nz * ny * nx;
    int64_t total = (int64_t)ceil(length / dt);
    if (k1 > total) k1 = total;
    if (k0 < 0 || k0 > k1) return EKGO_ERR_ARG;
    int64_t steps = k1 - k0;
    for (int64_t k = 0; k < k0; ++k) start += dt;
    int64_t *api = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int32_t *apl = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    double *apat = (double *)malloc((size_t)n * sizeof(double));
    int64_t na = ekgo_ap_indices(n, layer, at, api, apl, apat);
    ap_t *aps = (ap_t *)malloc((size_t)(na ? na : 1) * sizeof(ap_t));
    for (int64_t a = 0; a < na; ++a) ap_init(&aps[a], layer_k + 9 * (apl[a] - 1), apat[a]);
    int dif[26 * 3];
    int nnb = ekgo_neighbourhood(nhood_code, dif);
    double *cell = (double *)malloc((size_t)steps * sizeof(double));
    double *dip = (double *)malloc((size_t)steps * 3 * sizeof(double));
    for (int64_t i = 0; i < (int64_t)nlead * steps; ++i) ecg[i] = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        if (layer[i] <= 0) continue;
        int64_t z = i / ((int64_t)ny * nx), y = (i / nx) % ny, x = i % nx;
        const ap_t *ap = &aps[api[i]];
        double st = start;
        for (int64_t k = 0; k < steps; ++k) { cell[k] = ap_eval(ap, st); st += dt; }
        for (int64_t k = 0; k < 3 * steps; ++k) dip[k] = 0.0;
        for (int q = 0; q < nnb; ++q) {
            int64_t z2 = z - dif[3 * q], y2 = y - dif[3 * q + 1], x2 = x - dif[3 * q + 2];
            if (z2 < 0 || z2 >= nz || y2 < 0 || y2 >= ny || x2 < 0 || x2 >= nx) continue;
            int64_t j = (z2 * ny + y2) * nx + x2;
            if (layer[j] <= 0) continue;
            const ap_t *ap2 = &aps[api[j]];
            double st2 = start;
            for (int64_t k = 0; k < steps; ++k) {
                double vd = ap_eval(ap2, st2) - cell[k];
                dip[3 * k + 0] += (double)dif[3 * q + 0] * vd;
                dip[3 * k + 1] += (double)dif[3 * q + 1] * vd;
                dip[3 * k + 2] += (double)dif[3 * q + 2] * vd;
                st2 += dt;
            }
        }
        for (int l = 0; l < nlead; ++l) {
            double m0 = lead_zyx[3 * l + 0] - (double)(z + 1);
            double m1 = lead_zyx[3 * l + 1] - (double)(y + 1);
            double m2 = lead_zyx[3 * l + 2] - (double)(x + 1);
            double s = m0 * m0; s += m1 * m1; s += m2 * m2;
            double f = 1.0 / (s * sqrt(s));
            m0 *= f; m1 *= f; m2 *= f;
            for (int64_t k = 0; k < steps; ++k) {
                double r = 0.0;
                r += m0 * dip[3 * k]; r += m1 * dip[3 * k + 1]; r += m2 * dip[3 * k + 2];
                ecg[l * steps + k] += r;
            }
        }
    }
    free(dip); free(cell); free(aps); free(apat); free(apl); free(api);
    return EKGO_OK;
}

/* The whole time axis, or its first steps_limit steps. */
int ekgo_run_naive(int nz, int ny, int nx, const int32_t *layer, const double *at, int nlayers,
                   const double *layer_k, int nlead, const double *lead_zyx, int nhood_code, double start,
                   double length, double dt, int steps_limit, double *ecg) {
    int64_t steps = (int64_t)ceil(length / dt);
    if (steps_limit > 0 && steps_limit < steps) steps = steps_limit;
    return ekgo_run_naive_range(nz, ny, nx, layer, at, nlayers, layer_k, nlead, lead_zyx, nhood_code, start, length,
                                dt, 0, steps, ecg);
}
