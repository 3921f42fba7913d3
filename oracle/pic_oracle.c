/* pic_oracle.c -- TEST INFRASTRUCTURE ONLY (see pic_oracle.h).
 *
 * FP64 CPU restatement of the reference ch4/v3 PIC + DSMC step.  Each function cites the
 * reference file:line it follows.  Built by oracle/Makefile with -ffp-contract=off so that
 * the FP64 operation order written here is the one executed.
 */
#include "pic_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------ */
/* grid                                                                                   */
/* ------------------------------------------------------------------------------------ */

/* World::setExtents (World.cpp:63-78): dx = (xm-x0)/(nn-1), inv_dx = 1/dx */
void or_grid_init(or_grid* g, int ni, int nj, int nk, const double* x0, const double* xm, const int* periodic) {
    memset(g, 0, sizeof(*g));
    g->ni = ni;
    g->nj = nj;
    g->nk = nk;
    int nn[3] = {ni, nj, nk};
    for (int d = 0; d < 3; d++) {
        g->x0[d] = x0[d];
        g->xm[d] = xm[d];
        g->dx[d] = (xm[d] - x0[d]) / (nn[d] - 1);
        g->inv_dx[d] = 1 / g->dx[d];
        g->periodic[d] = periodic ? periodic[d] : 0;
    }
}

/* Rectangle(pos, phi, sides) (Object.h:103-104): half_sides = sides/2 */
int or_grid_add_box(or_grid* g, const double* center, const double* sides) {
    if (g->n_boxes >= 8) return -1;
    for (int d = 0; d < 3; d++) {
        g->box_c[g->n_boxes][d] = center[d];
        g->box_half[g->n_boxes][d] = sides[d] / 2;
    }
    return g->n_boxes++;
}

/* Rectangle::inObject (Object.cpp:231-238) over World::inObject (World.cpp:293-301) */
static int in_object(const or_grid* g, const double x[3]) {
    for (int b = 0; b < g->n_boxes; b++) {
        int in = 1;
        for (int d = 0; d < 3; d++)
            if (fabs(x[d] - g->box_c[b][d]) > g->box_half[b][d]) in = 0;
        if (in) return b + 1;
    }
    return 0;
}

static inline long U(const or_grid* g, int i, int j, int k) { return ((long)k * g->nj + j) * g->ni + i; }

void or_node_kinds(const or_grid* g, int wall_mode, uint8_t* kind) {
    int nn[3] = {g->ni, g->nj, g->nk};
    for (int k = 0; k < g->nk; k++)
        for (int j = 0; j < g->nj; j++)
            for (int i = 0; i < g->ni; i++) {
                int ijk[3] = {i, j, k};
                uint8_t kd = OR_FREE;
                int alias = 0, wall = 0;
                for (int d = 0; d < 3; d++) {
                    if (g->periodic[d] && ijk[d] == nn[d] - 1) alias = 1;
                    if (!g->periodic[d] && (ijk[d] == 0 || ijk[d] == nn[d] - 1)) wall = 1;
                }
                double x[3] = {g->x0[0] + i * g->dx[0], g->x0[1] + j * g->dx[1], g->x0[2] + k * g->dx[2]};
                if (alias) kd = OR_ALIAS;
                else if (in_object(g, x)) kd = OR_FIXED; /* World::computeObjectID, World.cpp:276-292 */
                else if (wall) kd = wall_mode == 1 ? OR_FIXED : OR_MIRROR;
                kind[U(g, i, j, k)] = kd;
            }
}

/* ------------------------------------------------------------------------------------ */
/* random numbers                                                                         */
/* ------------------------------------------------------------------------------------ */

/* MT19937 (Matsumoto & Nishimura 1998), the engine behind the reference's global Rnd
 * (Rnd.h:8, Rnd.cpp:7). */
void or_mt_seed(or_mt* r, uint32_t seed) {
    r->mt[0] = seed;
    for (int i = 1; i < 624; i++) r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->idx = 624;
}
uint32_t or_mt_next(or_mt* r) {
    if (r->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            uint32_t y = (r->mt[i] & 0x80000000u) | (r->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = r->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            r->mt[i] = v;
        }
        r->idx = 0;
    }
    uint32_t y = r->mt[r->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}
/* std::uniform_real_distribution<double>(0,1)(mt19937) as used by Rnd::operator()
 * (Rnd.cpp:10-12): generate_canonical<double,53> takes two 32-bit draws,
 * (g1 + g2*2^32) / 2^64, clamped below 1. */
double or_mt_u01(or_mt* r) {
    double sum = 0.0, tmp = 1.0;
    for (int k = 0; k < 2; k++) {
        sum += (double)or_mt_next(r) * tmp;
        tmp *= 4294967296.0;
    }
    double ret = sum / tmp;
    if (ret >= 1.0) ret = nextafter(1.0, 0.0);
    return 1.0 * ret + 0.0; /* (b-a)*u + a */
}
/* Rnd::operator()(min,max) (Rnd.cpp:13-15) */
static inline double mt_range(or_mt* r, double mn, double mx) { return mn + or_mt_u01(r) * (mx - mn); }

/* Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}
double or_u01_from_u32(uint32_t x) { return ((double)(x >> 9) + 0.5) * (1.0 / 8388608.0); }

/* splitmix64 finaliser (Steele, Lea, Flood 2014) */
static uint64_t or_mix64(uint64_t x) {
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
/* ids of collision products: the finaliser over parent id, step and product kind */
uint64_t or_child_id(uint64_t parent, uint32_t step, uint32_t kind) {
    return or_mix64(parent + 0x9E3779B97F4A7C15ull * ((((uint64_t)step) << 2) | (uint64_t)kind));
}
/* 32-bit draw of the null-collision candidate test: output step + 1 of a SplitMix64 stream
 * seeded by the scrambled (id xor seed) */
uint32_t or_cand_draw(uint64_t id, uint32_t step, uint32_t seed_lo, uint32_t seed_hi) {
    uint64_t s = or_mix64(id ^ (((uint64_t)seed_hi << 32) | seed_lo));
    return (uint32_t)(or_mix64(s + 0x9E3779B97F4A7C15ull * ((uint64_t)step + 1ull)) >> 32);
}
/* candidate iff draw < T, T = floor(p 2^32) clamped to [0, 2^32 - 1] */
uint32_t or_cand_threshold(double p) {
    if (!(p > 0.0)) return 0u;
    if (p >= 1.0) return 0xFFFFFFFFu;
    return (uint32_t)(p * 4294967296.0);
}

/* ------------------------------------------------------------------------------------ */
/* fields                                                                                 */
/* ------------------------------------------------------------------------------------ */

/* World::computeNodeVolumes (World.cpp:353-366); a periodic axis has no boundary faces. */
void or_node_volumes(const or_grid* g, double* vol) {
    double base = g->dx[0] * g->dx[1] * g->dx[2];
    int nn[3] = {g->ni, g->nj, g->nk};
    for (int k = 0; k < g->nk; k++)
        for (int j = 0; j < g->nj; j++)
            for (int i = 0; i < g->ni; i++) {
                int ijk[3] = {i, j, k};
                double v = base;
                for (int d = 0; d < 3; d++)
                    if (!g->periodic[d] && (ijk[d] == 0 || ijk[d] == nn[d] - 1)) v *= 0.5;
                vol[U(g, i, j, k)] = v;
            }
}

/* World::XtoL (World.cpp:123-128) */
static inline void xtol(const or_grid* g, const double x[3], double lc[3]) {
    for (int d = 0; d < 3; d++) lc[d] = (x[d] - g->x0[d]) * g->inv_dx[d];
}

/* Field<Vec3>::gather (Field.h:200-232), same term order; f3 is node-major xyz. */
void or_gather3_ref(const or_grid* g, const double* f3, const double lc[3], double out[3]) {
    int i = (int)lc[0], j = (int)lc[1], k = (int)lc[2];
    double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
    double one_dj = 1 - dj, one_di = 1 - di, one_dk = 1 - dk;
    double w_ij = one_di * one_dj, w_ij1 = one_di * dj, w_i1j = di * one_dj, w_i1j1 = di * dj;
    long n_ij = U(g, i, j, k), n_ij1 = U(g, i, j + 1, k), n_i1j = U(g, i + 1, j, k), n_i1j1 = U(g, i + 1, j + 1, k);
    long sk = (long)g->ni * g->nj;
    for (int d = 0; d < 3; d++) {
        double v = f3[3 * n_ij + d] * w_ij * one_dk;
        v = v + f3[3 * (n_ij + sk) + d] * w_ij * dk;
        v = v + f3[3 * n_ij1 + d] * w_ij1 * one_dk;
        v = v + f3[3 * (n_ij1 + sk) + d] * w_ij1 * dk;
        v = v + f3[3 * n_i1j + d] * w_i1j * one_dk;
        v = v + f3[3 * (n_i1j + sk) + d] * w_i1j * dk;
        v = v + f3[3 * n_i1j1 + d] * w_i1j1 * one_dk;
        v = v + f3[3 * (n_i1j1 + sk) + d] * w_i1j1 * dk;
        out[d] = v;
    }
}

/* Field<double>::scatter (Field.h:156-199), same operation order. */
void or_scatter_ref(const or_grid* g, double* f, const double lc[3], double val) {
    int i = (int)lc[0], j = (int)lc[1], k = (int)lc[2];
    double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
    double one_di = 1 - di, one_dj = 1 - dj, one_dk = 1 - dk;
    double a = val * one_di * one_dj, b = val * one_di * dj, c = val * di * one_dj, e = val * di * dj;
    long sk = (long)g->ni * g->nj;
    long n_ij = U(g, i, j, k), n_ij1 = U(g, i, j + 1, k), n_i1j = U(g, i + 1, j, k), n_i1j1 = U(g, i + 1, j + 1, k);
    f[n_ij] += a * one_dk;
    f[n_ij + sk] += a * dk;
    f[n_ij1] += b * one_dk;
    f[n_ij1 + sk] += b * dk;
    f[n_i1j] += c * one_dk;
    f[n_i1j + sk] += c * dk;
    f[n_i1j1] += e * one_dk;
    f[n_i1j1 + sk] += e * dk;
}

/* fold the copy at index n-1 of every periodic axis onto index 0 and mirror it back */
static void fold_periodic(const or_grid* g, double* f) {
    int ni = g->ni, nj = g->nj, nk = g->nk;
    if (g->periodic[0])
        for (int k = 0; k < nk; k++)
            for (int j = 0; j < nj; j++) {
                f[U(g, 0, j, k)] += f[U(g, ni - 1, j, k)];
                f[U(g, ni - 1, j, k)] = f[U(g, 0, j, k)];
            }
    if (g->periodic[1])
        for (int k = 0; k < nk; k++)
            for (int i = 0; i < ni; i++) {
                f[U(g, i, 0, k)] += f[U(g, i, nj - 1, k)];
                f[U(g, i, nj - 1, k)] = f[U(g, i, 0, k)];
            }
    if (g->periodic[2])
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                f[U(g, i, j, 0)] += f[U(g, i, j, nk - 1)];
                f[U(g, i, j, nk - 1)] = f[U(g, i, j, 0)];
            }
}

/* Species::computeNumberDensity (Species.cpp:401-416): clear, scatter weights, den /= node_vol */
void or_number_density_ref(const or_grid* g, const or_particle* p, long n, double* den) {
    long nv = (long)g->ni * g->nj * g->nk;
    memset(den, 0, sizeof(double) * nv);
    for (long q = 0; q < n; q++) {
        double lc[3];
        xtol(g, p[q].pos, lc);
        or_scatter_ref(g, den, lc, p[q].w);
    }
    fold_periodic(g, den);
    double* vol = (double*)malloc(sizeof(double) * nv);
    or_node_volumes(g, vol);
    for (long q = 0; q < nv; q++) den[q] /= vol[q];
    free(vol);
}

/* PotentialSolver::computeEF (PotentialSolver.cpp:354-408).  Periodic axes use central
 * differences across the seam (index 0 sees n-2 and 1); the copy at n-1 equals index 0. */
void or_compute_ef_ref(const or_grid* g, const double* phi, double* ef) {
    int nn[3] = {g->ni, g->nj, g->nk};
    long st[3] = {1, g->ni, (long)g->ni * g->nj};
    double inv2[3];
    for (int d = 0; d < 3; d++) inv2[d] = 1.0 / (2 * g->dx[d]);
    for (int k = 0; k < g->nk; k++)
        for (int j = 0; j < g->nj; j++)
            for (int i = 0; i < g->ni; i++) {
                int ijk[3] = {i, j, k};
                long n = U(g, i, j, k);
                for (int d = 0; d < 3; d++) {
                    int c = ijk[d];
                    double e;
                    if (g->periodic[d]) {
                        int cc = (c == nn[d] - 1) ? 0 : c;
                        long base = n - (long)(c - cc) * st[d];
                        long im = base + (long)((cc == 0 ? nn[d] - 2 : cc - 1) - cc) * st[d];
                        long ip = base + (long)((cc + 1 == nn[d] - 1 ? 0 : cc + 1) - cc) * st[d];
                        e = (phi[im] - phi[ip]) * inv2[d];
                    } else if (nn[d] == 2) {
                        /* one cell: first-order difference (the reference would read past the end) */
                        e = c == 0 ? 2.0 * (phi[n] - phi[n + st[d]]) * inv2[d] : 2.0 * (phi[n - st[d]] - phi[n]) * inv2[d];
                    } else if (c == 0) {
                        e = (3 * phi[n] - 4 * phi[n + st[d]] + phi[n + 2 * st[d]]) * inv2[d];
                    } else if (c == nn[d] - 1) {
                        e = (-phi[n - 2 * st[d]] + 4 * phi[n - st[d]] - 3 * phi[n]) * inv2[d];
                    } else {
                        e = (phi[n - st[d]] - phi[n + st[d]]) * inv2[d];
                    }
                    ef[3 * n + d] = e;
                }
            }
}

/* ------------------------------------------------------------------------------------ */
/* push                                                                                   */
/* ------------------------------------------------------------------------------------ */

/* one particle of Species::advanceElectronsSerial (Species.cpp:369-388); returns 0 to delete.
 * Periodic axes (absent in the reference) wrap the position instead of deleting. */
static int push_one(const or_grid* g, or_particle* part, const double* ef, double dt, double factor) {
    double lc[3], e[3];
    xtol(g, part->pos, lc);
    or_gather3_ref(g, ef, lc, e);
    for (int d = 0; d < 3; d++) part->vel[d] += e[d] * factor;
    for (int d = 0; d < 3; d++) part->pos[d] += part->vel[d] * dt;
    for (int d = 0; d < 3; d++) {
        if (!g->periodic[d]) continue;
        double L = g->xm[d] - g->x0[d];
        if (part->pos[d] < g->x0[d]) part->pos[d] += L;
        else if (part->pos[d] >= g->xm[d]) part->pos[d] -= L;
    }
    if (in_object(g, part->pos)) return 0;
    for (int d = 0; d < 3; d++) /* World::inBounds (World.cpp:201-205) */
        if (part->pos[d] < g->x0[d] || part->pos[d] >= g->xm[d]) return 0;
    return 1;
}

/* Species::advanceElectronsSerial (Species.cpp:356-399): swap-with-last deletion. */
long or_push_electrons_ref(const or_grid* g, or_particle* p, long n, uint64_t* ids, const double* ef, double dt,
                           double charge, double mass) {
    double factor = dt * charge / mass;
    long np = n;
    for (long q = 0; q < np; q++) {
        if (!push_one(g, &p[q], ef, dt, factor)) {
            p[q] = p[np - 1];
            if (ids) ids[q] = ids[np - 1];
            np--;
            q--;
        }
    }
    return np;
}

typedef struct {
    const or_grid* g;
    or_particle* p;
    const double* ef;
    double dt, factor;
    long start, stop;
    long* dead;
    long n_dead;
} push_task;
static void* push_worker(void* arg) {
    push_task* t = (push_task*)arg;
    t->n_dead = 0;
    for (long q = t->start; q < t->stop; q++)
        if (!push_one(t->g, &t->p[q], t->ef, t->dt, t->factor)) t->dead[t->n_dead++] = q;
    return NULL;
}
static int cmp_desc(const void* a, const void* b) {
    long x = *(const long*)a, y = *(const long*)b;
    return (x < y) - (x > y);
}
/* Species::advanceElectrons multithreaded branch (Species.cpp:263-309) with the deletion
 * buffers actually filled (the reference passes copies through std::bind and loses them):
 * chunks per splitIntoChunks (Config.cpp:79-99), then descending swap-with-last deletion. */
long or_push_electrons_mt(const or_grid* g, or_particle* p, long n, uint64_t* ids, const double* ef, double dt,
                          double charge, double mass, int nthreads) {
    if (nthreads <= 1 || n < nthreads) return or_push_electrons_ref(g, p, n, ids, ef, dt, charge, mass);
    double factor = dt * charge / mass;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    push_task* tk = (push_task*)malloc(sizeof(push_task) * nthreads);
    long base = n / nthreads, extra = n % nthreads, s = 0;
    for (int t = 0; t < nthreads; t++) {
        long len = base + (t < extra ? 1 : 0);
        tk[t] = (push_task){g, p, ef, dt, factor, s, s + len, (long*)malloc(sizeof(long) * (len + 1)), 0};
        s += len;
        pthread_create(&th[t], NULL, push_worker, &tk[t]);
    }
    long total = 0;
    for (int t = 0; t < nthreads; t++) {
        pthread_join(th[t], NULL);
        total += tk[t].n_dead;
    }
    long* all = (long*)malloc(sizeof(long) * (total + 1));
    long m = 0;
    for (int t = 0; t < nthreads; t++) {
        memcpy(all + m, tk[t].dead, sizeof(long) * tk[t].n_dead);
        m += tk[t].n_dead;
        free(tk[t].dead);
    }
    qsort(all, total, sizeof(long), cmp_desc);
    long last = n - 1;
    for (long q = 0; q < total; q++) {
        p[all[q]] = p[last];
        if (ids) ids[all[q]] = ids[last];
        last--;
    }
    free(all);
    free(tk);
    free(th);
    return n - total;
}

/* ------------------------------------------------------------------------------------ */
/* Poisson                                                                                */
/* ------------------------------------------------------------------------------------ */

/* neighbour index along axis d (0,1,2) in direction s (-1,+1) with periodic wrap;
 * returns -1 outside a non-periodic domain. */
static inline long nb_index(const or_grid* g, int i, int j, int k, int d, int s) {
    int nn[3] = {g->ni, g->nj, g->nk};
    int ijk[3] = {i, j, k};
    int c = ijk[d] + s;
    if (g->periodic[d]) {
        if (c < 0) c = nn[d] - 2;
        else if (c >= nn[d] - 1) c = 0;
    } else if (c < 0 || c >= nn[d])
        return -1;
    ijk[d] = c;
    return U(g, ijk[0], ijk[1], ijk[2]);
}
/* the node a wall node copies in the reference GS (PotentialSolver.cpp:96-107): priority
 * i==0, i==ni-1, j==0, j==nj-1, k==0, k==nk-1 */
static long mirror_src(const or_grid* g, int i, int j, int k) {
    if (i == 0) return U(g, i + 1, j, k);
    if (i == g->ni - 1) return U(g, i - 1, j, k);
    if (j == 0) return U(g, i, j + 1, k);
    if (j == g->nj - 1) return U(g, i, j - 1, k);
    if (k == 0) return U(g, i, j, k + 1);
    return U(g, i, j, k - 1);
}
static long alias_src(const or_grid* g, int i, int j, int k) {
    if (g->periodic[0] && i == g->ni - 1) i = 0;
    if (g->periodic[1] && j == g->nj - 1) j = 0;
    if (g->periodic[2] && k == g->nk - 1) k = 0;
    return U(g, i, j, k);
}

/* PotentialSolver::solveGS (PotentialSolver.cpp:69-166), v3 semantics generalised by node
 * kind: FIXED skipped (object_id>0), MIRROR copies as the reference walls do, FREE gets the
 * SOR update with omega = 1.4; residual check every 25 sweeps, L2 = sqrt(sum R^2 / nv).
 * With every wall FIXED this is also ch2's Dirichlet GS (ch2/v1/PotentialSolver.cpp:37-72). */
int or_solve_gs_ref(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, int max_it, double tol,
                    int* iters, double* l2) {
    const double SOR = 1.4;
    double inv_d2x = 1.0 / (g->dx[0] * g->dx[0]), inv_d2y = 1.0 / (g->dx[1] * g->dx[1]),
           inv_d2z = 1.0 / (g->dx[2] * g->dx[2]);
    double inv_eps0 = 1.0 / OR_EPS0;
    double twos = 2.0 * (inv_d2x + inv_d2y + inv_d2z);
    double inv_twos = 1.0 / twos;
    long nv = (long)g->ni * g->nj * g->nk;
    double L2 = 0;
    int converged = 0, it;
    for (it = 0; it < max_it; it++) {
        for (int i = 0; i < g->ni; i++)
            for (int j = 0; j < g->nj; j++)
                for (int k = 0; k < g->nk; k++) {
                    long n = U(g, i, j, k);
                    uint8_t kd = kind[n];
                    if (kd == OR_FIXED) continue;
                    if (kd == OR_MIRROR) {
                        phi[n] = phi[mirror_src(g, i, j, k)];
                        continue;
                    }
                    if (kd == OR_ALIAS) {
                        phi[n] = phi[alias_src(g, i, j, k)];
                        continue;
                    }
                    double new_phi = (rho[n] * inv_eps0 +
                                      (phi[nb_index(g, i, j, k, 0, -1)] + phi[nb_index(g, i, j, k, 0, 1)]) * inv_d2x +
                                      (phi[nb_index(g, i, j, k, 1, -1)] + phi[nb_index(g, i, j, k, 1, 1)]) * inv_d2y +
                                      (phi[nb_index(g, i, j, k, 2, -1)] + phi[nb_index(g, i, j, k, 2, 1)]) * inv_d2z) *
                                     inv_twos;
                    phi[n] = phi[n] + SOR * (new_phi - phi[n]);
                }
        if (it % 25 == 0) {
            double sum = 0;
            for (int i = 0; i < g->ni; i++)
                for (int j = 0; j < g->nj; j++)
                    for (int k = 0; k < g->nk; k++) {
                        long n = U(g, i, j, k);
                        uint8_t kd = kind[n];
                        double R;
                        if (kd == OR_FIXED) continue;
                        if (kd == OR_MIRROR) R = phi[n] - phi[mirror_src(g, i, j, k)];
                        else if (kd == OR_ALIAS) R = phi[n] - phi[alias_src(g, i, j, k)];
                        else
                            R = -phi[n] * twos + rho[n] * inv_eps0 +
                                (phi[nb_index(g, i, j, k, 0, -1)] + phi[nb_index(g, i, j, k, 0, 1)]) * inv_d2x +
                                (phi[nb_index(g, i, j, k, 1, -1)] + phi[nb_index(g, i, j, k, 1, 1)]) * inv_d2y +
                                (phi[nb_index(g, i, j, k, 2, -1)] + phi[nb_index(g, i, j, k, 2, 1)]) * inv_d2z;
                        sum += R * R;
                    }
            L2 = sqrt(sum / nv);
            if (L2 < tol) {
                converged = 1;
                break;
            }
        }
    }
    if (iters) *iters = converged ? it + 1 : it;
    if (l2) *l2 = L2;
    return converged;
}

/* ---- reference NR-PCG restated on its 7-slot row matrix ---- */
typedef struct {
    double a[7];
    long col[7];
    int n;
} row7;
static inline void row_set(row7* r, long c, double v) {
    for (int s = 0; s < r->n; s++)
        if (r->col[s] == c) {
            r->a[s] = v;
            return;
        }
    r->col[r->n] = c;
    r->a[r->n] = v;
    r->n++;
}
static inline double row_get(const row7* r, long c) {
    for (int s = 0; s < r->n; s++)
        if (r->col[s] == c) return r->a[s];
    return 0;
}
/* Matrix::operator* (Matrix.cpp:117-141): slot order as inserted */
static void spmv7(const row7* A, const double* v, double* out, long n) {
    for (long u = 0; u < n; u++) {
        double s = 0;
        for (int q = 0; q < A[u].n; q++) s += A[u].a[q] * v[A[u].col[q]];
        out[u] = s;
    }
}
static double dot(const double* a, const double* b, long n) { /* operator*(tcvector,tcvector), Matrix.cpp:257 */
    double r = 0;
    for (long i = 0; i < n; i++) r += a[i] * b[i];
    return r;
}
/* vec::norm (PotentialSolver.cpp:36-38): RMS */
static double rms(const double* a, long n) { return sqrt(dot(a, a, n) / n); }

/* PotentialSolver::buildMatrix (PotentialSolver.cpp:414-471).  axis_swap=1 keeps the
 * reference's coefficient assignment (k-neighbours get 1/dx^2, i-neighbours 1/dz^2,
 * lines 457-463); axis_swap=0 gives each axis its own coefficient. */
static void build_matrix_ref(const or_grid* g, const uint8_t* kind, row7* A, int* ntype, int axis_swap) {
    double inv_d2x = 1.0 / (g->dx[0] * g->dx[0]), inv_d2y = 1.0 / (g->dx[1] * g->dx[1]),
           inv_d2z = 1.0 / (g->dx[2] * g->dx[2]);
    double twos = 2.0 * (inv_d2x + inv_d2y + inv_d2z);
    double inv_dx = 1.0 / g->dx[0], inv_dy = 1.0 / g->dx[1], inv_dz = 1.0 / g->dx[2];
    double ck = axis_swap ? inv_d2x : inv_d2z, ci = axis_swap ? inv_d2z : inv_d2x;
    long ni = g->ni, ninj = (long)g->ni * g->nj;
    for (int k = 0; k < g->nk; k++)
        for (int j = 0; j < g->nj; j++)
            for (int i = 0; i < g->ni; i++) {
                long u = U(g, i, j, k);
                A[u].n = 0;
                uint8_t kd = kind[u];
                if (kd == OR_FIXED) {
                    row_set(&A[u], u, 1);
                    ntype[u] = 2; /* DIRICHLET */
                    continue;
                }
                ntype[u] = 1; /* NEUMANN */
                if (kd == OR_ALIAS) {
                    row_set(&A[u], u, 1);
                    row_set(&A[u], alias_src(g, i, j, k), -1);
                } else if (kd == OR_MIRROR) {
                    if (i == 0) {
                        row_set(&A[u], u, inv_dx);
                        row_set(&A[u], u + 1, -inv_dx);
                    } else if (i == g->ni - 1) {
                        row_set(&A[u], u, inv_dx);
                        row_set(&A[u], u - 1, -inv_dx);
                    } else if (j == 0) {
                        row_set(&A[u], u, inv_dy);
                        row_set(&A[u], u + ni, -inv_dy);
                    } else if (j == g->nj - 1) {
                        row_set(&A[u], u, inv_dy);
                        row_set(&A[u], u - ni, -inv_dy);
                    } else if (k == 0) {
                        row_set(&A[u], u, inv_dz);
                        row_set(&A[u], u + ninj, -inv_dz);
                    } else {
                        row_set(&A[u], u, inv_dz);
                        row_set(&A[u], u - ninj, -inv_dz);
                    }
                } else {
                    ntype[u] = 0; /* REGULAR */
                    row_set(&A[u], nb_index(g, i, j, k, 2, -1), ck);
                    row_set(&A[u], nb_index(g, i, j, k, 1, -1), inv_d2y);
                    row_set(&A[u], nb_index(g, i, j, k, 0, -1), ci);
                    row_set(&A[u], u, -twos);
                    row_set(&A[u], nb_index(g, i, j, k, 0, 1), ci);
                    row_set(&A[u], nb_index(g, i, j, k, 1, 1), inv_d2y);
                    row_set(&A[u], nb_index(g, i, j, k, 2, 1), ck);
                }
            }
}

/* PotentialSolver::solveGSlinear (PotentialSolver.cpp:315-347) */
static int gs_linear(const row7* A, double* x, const double* b, long n, int max_it, double tol) {
    double* R = (double*)malloc(sizeof(double) * n);
    int conv = 0;
    for (int it = 0; it < max_it; it++) {
        for (long i = 0; i < n; i++) {
            double S = 0;
            for (int q = 0; q < A[i].n; q++) S += A[i].a[q] * x[A[i].col[q]];
            double aii = row_get(&A[i], i);
            S = S - aii * x[i];
            double phi_new = (b[i] - S) / aii;
            x[i] = x[i] + 1.0 * (phi_new - x[i]);
        }
        if (it % 25 == 0) {
            spmv7(A, x, R, n);
            for (long i = 0; i < n; i++) R[i] = R[i] - b[i];
            if (rms(R, n) < tol) {
                conv = 1;
                break;
            }
        }
    }
    free(R);
    return conv;
}

/* PotentialSolver::solveNRPCG + solvePCGlinear (PotentialSolver.cpp:178-313) with n0 = 0
 * (main.cpp:138), where the Newton Jacobian is the matrix itself. */
int or_solve_pcg_ref(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, int max_it, double tol,
                     int axis_swap, int* iters, double* l2) {
    long n = (long)g->ni * g->nj * g->nk;
    row7* A = (row7*)calloc(n, sizeof(row7));
    int* ntype = (int*)malloc(sizeof(int) * n);
    build_matrix_ref(g, kind, A, ntype, axis_swap);
    double* Minv = (double*)malloc(sizeof(double) * n);
    for (long u = 0; u < n; u++) Minv[u] = 1 / row_get(&A[u], u); /* Matrix::invDiagonal */
    double inv_eps0 = 1.0 / OR_EPS0;
    double *b = (double*)malloc(sizeof(double) * n), *y = (double*)calloc(n, sizeof(double)),
           *F = (double*)malloc(sizeof(double) * n), *gv = (double*)malloc(sizeof(double) * n),
           *s = (double*)malloc(sizeof(double) * n), *d = (double*)malloc(sizeof(double) * n),
           *z = (double*)malloc(sizeof(double) * n);
    for (long u = 0; u < n; u++) {
        if (ntype[u] == 1) b[u] = 0;
        else if (ntype[u] == 2) b[u] = phi[u];
        else b[u] = -rho[u] * inv_eps0;
    }
    int converged = 0, total_it = 0, status = 0;
    double L2 = 0;
    for (int nr = 0; nr < 20 && status == 0; nr++) {
        spmv7(A, phi, F, n);
        for (long u = 0; u < n; u++) F[u] = F[u] - b[u];
        /* solvePCGlinear(J=A, y, F) */
        int pconv = 0;
        spmv7(A, y, gv, n);
        for (long u = 0; u < n; u++) gv[u] = gv[u] - F[u];
        for (long u = 0; u < n; u++) s[u] = gv[u] * Minv[u];
        for (long u = 0; u < n; u++) d[u] = s[u] * -1;
        for (int it = 0; it < max_it; it++) {
            spmv7(A, d, z, n);
            double alpha = dot(gv, s, n);
            double beta = dot(d, z, n);
            total_it++;
            if (beta == 0) {
                status = -1;
                break;
            }
            for (long u = 0; u < n; u++) y[u] = y[u] + d[u] * (alpha / beta);
            for (long u = 0; u < n; u++) gv[u] = gv[u] + z[u] * (alpha / beta);
            for (long u = 0; u < n; u++) s[u] = gv[u] * Minv[u];
            beta = alpha;
            alpha = dot(gv, s, n);
            for (long u = 0; u < n; u++) d[u] = d[u] * (alpha / beta) - s[u];
            L2 = rms(gv, n);
            if (L2 < tol) {
                pconv = 1;
                break;
            }
        }
        if (status) break;
        if (!pconv) gs_linear(A, y, F, n, 20 * max_it, tol);
        for (long u = 0; u < n; u++)
            if (ntype[u] == 2) y[u] = 0;
        for (long u = 0; u < n; u++) phi[u] = phi[u] - y[u];
        if (rms(y, n) < 1e-3) {
            converged = 1;
            break;
        }
    }
    free(A);
    free(ntype);
    free(Minv);
    free(b);
    free(y);
    free(F);
    free(gv);
    free(s);
    free(d);
    free(z);
    if (iters) *iters = total_it;
    if (l2) *l2 = L2;
    return status ? status : converged;
}

/* ---- GPU-form Poisson on the reduced system (restatement of the CUDA kernels) ----
 * For a FREE node p and each face neighbour q (periodic wrap applied):
 *   FREE q  -> off-diagonal -c_d * phi_q
 *   FIXED q -> known value moved to the right-hand side
 *   MIRROR q-> equals phi_p (the reference walls copy their inner neighbour): no term,
 *              and c_d is left out of the diagonal.
 * L phi = rho/eps0, L symmetric positive definite when at least one FIXED node exists. */
static void node_ijk(const or_grid* g, long n, int* i, int* j, int* k) {
    *i = (int)(n % g->ni);
    *j = (int)((n / g->ni) % g->nj);
    *k = (int)(n / ((long)g->ni * g->nj));
}
/* y = L x restricted to FREE nodes; FIXED neighbours contribute fixed_scale*x_q */
static void apply_L(const or_grid* g, const uint8_t* kind, const double* x, double* y, int fixed_as_zero) {
    long nv = (long)g->ni * g->nj * g->nk;
    double c[3];
    for (int d = 0; d < 3; d++) c[d] = 1.0 / (g->dx[d] * g->dx[d]);
    for (long n = 0; n < nv; n++) {
        if (kind[n] != OR_FREE) {
            y[n] = 0;
            continue;
        }
        int i, j, k;
        node_ijk(g, n, &i, &j, &k);
        double diag = 0, off = 0;
        for (int d = 0; d < 3; d++)
            for (int s = -1; s <= 1; s += 2) {
                long q = nb_index(g, i, j, k, d, s);
                uint8_t kq = kind[q];
                if (kq == OR_MIRROR) continue;
                diag += c[d];
                if (kq == OR_FREE) off += c[d] * x[q];
                else if (!fixed_as_zero) off += c[d] * x[q];
            }
        y[n] = diag * x[n] - off;
    }
}
static double diag_of(const or_grid* g, const uint8_t* kind, long n) {
    int i, j, k;
    node_ijk(g, n, &i, &j, &k);
    double diag = 0;
    for (int d = 0; d < 3; d++)
        for (int s = -1; s <= 1; s += 2)
            if (kind[nb_index(g, i, j, k, d, s)] != OR_MIRROR) diag += 1.0 / (g->dx[d] * g->dx[d]);
    return diag;
}
void or_residual(const or_grid* g, const uint8_t* kind, const double* phi, const double* rho, double* rnorm2,
                 double* bnorm2) {
    long nv = (long)g->ni * g->nj * g->nk;
    double* Lx = (double*)malloc(sizeof(double) * nv);
    double* Lf = (double*)malloc(sizeof(double) * nv);
    apply_L(g, kind, phi, Lx, 0);
    apply_L(g, kind, phi, Lf, 1); /* Lf - Lx = -(fixed neighbour terms) */
    double r2 = 0, b2 = 0;
    for (long n = 0; n < nv; n++) {
        if (kind[n] != OR_FREE) continue;
        double b = rho[n] / OR_EPS0 + (Lf[n] - Lx[n]);
        double r = b - Lf[n];
        r2 += r * r;
        b2 += b * b;
    }
    free(Lx);
    free(Lf);
    *rnorm2 = r2;
    *bnorm2 = b2;
}
/* MIRROR nodes take the clamped interior value, ALIAS nodes their periodic source. */
void or_fill_aux(const or_grid* g, const uint8_t* kind, double* phi) {
    long nv = (long)g->ni * g->nj * g->nk;
    for (long n = 0; n < nv; n++) {
        int i, j, k;
        node_ijk(g, n, &i, &j, &k);
        if (kind[n] == OR_MIRROR) {
            int ci = i, cj = j, ck = k;
            if (!g->periodic[0]) ci = ci < 1 ? 1 : (ci > g->ni - 2 ? g->ni - 2 : ci);
            if (!g->periodic[1]) cj = cj < 1 ? 1 : (cj > g->nj - 2 ? g->nj - 2 : cj);
            if (!g->periodic[2]) ck = ck < 1 ? 1 : (ck > g->nk - 2 ? g->nk - 2 : ck);
            phi[n] = phi[U(g, ci, cj, ck)];
        }
    }
    for (long n = 0; n < nv; n++)
        if (kind[n] == OR_ALIAS) {
            int i, j, k;
            node_ijk(g, n, &i, &j, &k);
            phi[n] = phi[alias_src(g, i, j, k)];
        }
}
/* red-black SOR on the reduced system, colour (i+j+k)&1, checked every 10 sweeps */
int or_solve_rbsor(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, double omega, double tol_rel,
                   int max_sweeps, int* sweeps, double* rel) {
    long nv = (long)g->ni * g->nj * g->nk;
    double c[3];
    for (int d = 0; d < 3; d++) c[d] = 1.0 / (g->dx[d] * g->dx[d]);
    int conv = 0, s;
    double r2, b2, rr = 1;
    for (s = 0; s < max_sweeps; s++) {
        for (int color = 0; color < 2; color++)
            for (long n = 0; n < nv; n++) {
                if (kind[n] != OR_FREE) continue;
                int i, j, k;
                node_ijk(g, n, &i, &j, &k);
                if (((i + j + k) & 1) != color) continue;
                double diag = 0, off = 0;
                for (int d = 0; d < 3; d++)
                    for (int sg = -1; sg <= 1; sg += 2) {
                        long q = nb_index(g, i, j, k, d, sg);
                        if (kind[q] == OR_MIRROR) continue;
                        diag += c[d];
                        off += c[d] * phi[q];
                    }
                double gsv = (rho[n] / OR_EPS0 + off) / diag;
                phi[n] += omega * (gsv - phi[n]);
            }
        if ((s + 1) % 10 == 0 || s + 1 == max_sweeps) {
            or_residual(g, kind, phi, rho, &r2, &b2);
            rr = b2 > 0 ? sqrt(r2 / b2) : sqrt(r2);
            if (rr <= tol_rel) {
                conv = 1;
                s++;
                break;
            }
        }
    }
    or_fill_aux(g, kind, phi);
    if (sweeps) *sweeps = s;
    if (rel) *rel = rr;
    return conv;
}
/* flexible (Polak-Ribiere) Jacobi-preconditioned CG on the reduced system */
int or_solve_fpcg(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, double tol_rel, int max_it,
                  int* iters, double* rel) {
    long nv = (long)g->ni * g->nj * g->nk;
    double *r = (double*)calloc(nv, sizeof(double)), *z = (double*)calloc(nv, sizeof(double)),
           *d = (double*)calloc(nv, sizeof(double)), *q = (double*)calloc(nv, sizeof(double)),
           *dg = (double*)calloc(nv, sizeof(double)), *Lf = (double*)calloc(nv, sizeof(double));
    double r2, b2;
    apply_L(g, kind, phi, q, 0);
    apply_L(g, kind, phi, Lf, 1);
    b2 = 0;
    for (long n = 0; n < nv; n++) {
        if (kind[n] != OR_FREE) continue;
        double b = rho[n] / OR_EPS0 + (Lf[n] - q[n]);
        r[n] = b - Lf[n];
        b2 += b * b;
        dg[n] = diag_of(g, kind, n);
        z[n] = r[n] / dg[n];
        d[n] = z[n];
    }
    double rz = 0;
    r2 = 0;
    for (long n = 0; n < nv; n++) {
        rz += r[n] * z[n];
        r2 += r[n] * r[n];
    }
    double bn = b2 > 0 ? sqrt(b2) : 1;
    int it = 0, conv = sqrt(r2) / bn <= tol_rel;
    while (!conv && it < max_it) {
        apply_L(g, kind, d, q, 1);
        double dq = dot(d, q, nv);
        if (dq == 0) break;
        double alpha = rz / dq;
        double rzo = 0, rzn = 0;
        r2 = 0;
        for (long n = 0; n < nv; n++) {
            if (kind[n] != OR_FREE) continue;
            phi[n] += alpha * d[n];
            r[n] -= alpha * q[n];
            double zn = r[n] / dg[n];
            rzo += r[n] * z[n];
            rzn += r[n] * zn;
            z[n] = zn;
            r2 += r[n] * r[n];
        }
        it++;
        if (sqrt(r2) / bn <= tol_rel) {
            conv = 1;
            break;
        }
        double beta = (rzn - rzo) / rz;
        rz = rzn;
        for (long n = 0; n < nv; n++)
            if (kind[n] == OR_FREE) d[n] = z[n] + beta * d[n];
    }
    or_fill_aux(g, kind, phi);
    if (iters) *iters = it;
    if (rel) *rel = sqrt(r2) / bn;
    free(r);
    free(z);
    free(d);
    free(q);
    free(dg);
    free(Lf);
    return conv;
}

/* ------------------------------------------------------------------------------------ */
/* collisions                                                                             */
/* ------------------------------------------------------------------------------------ */

/* MC_MEX_Ionization::evaluateSigmaColl (Interactions.cpp:541-558): std::map::lower_bound
 * (first key >= E), clamp at both ends, linear interpolation otherwise. */
double or_sigma_coll(const or_coll_params* cp, double E) {
    const double* x = cp->table_E;
    int n = cp->table_n, lo = 0, hi = n; /* first index with x >= E */
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (x[mid] < E) lo = mid + 1;
        else hi = mid;
    }
    if (lo == 0) return cp->table_s[0];
    if (lo == n) return cp->table_s[n - 1];
    double x1 = x[lo - 1], x2 = x[lo], y1 = cp->table_s[lo - 1], y2 = cp->table_s[lo];
    return y1 + (E - x1) * (y2 - y1) / (x2 - x1);
}
/* MC_MEX_Ionization::evaluateSigmaIon (Interactions.cpp:559-566) and the Lotz form */
double or_sigma_ion(const or_coll_params* cp, double E) {
    if (E <= cp->E_ion_eV) return 0;
    if (cp->sigma_ion_kind == 0) return cp->sig_a * log(E / cp->sig_b) / E * exp(-cp->sig_c / E);
    double I = cp->E_ion_eV, x = E / I;
    return cp->sig_A * log(x) / (E * I) * (1 - cp->sig_b * exp(-cp->sig_c * (x - 1)));
}
/* max over the table range of sigma_coll(E)*v_rel(E), v_rel = sqrt(2 E q / m_red): on each
 * linear segment the maximum of (a + bE) sqrt(E) is at an end or at E = -a/(3b). */
double or_sigv_majorant(const or_coll_params* cp) {
    double m_red = cp->mass_neutral * cp->mass_electron / (cp->mass_neutral + cp->mass_electron);
    double best = 0;
    for (int s = 0; s < cp->table_n; s++) {
        double E = cp->table_E[s];
        double v = sqrt(2 * E * OR_QE / m_red) * cp->table_s[s];
        if (v > best) best = v;
        if (s + 1 < cp->table_n) {
            double x1 = cp->table_E[s], x2 = cp->table_E[s + 1], y1 = cp->table_s[s], y2 = cp->table_s[s + 1];
            double b = (y2 - y1) / (x2 - x1), a = y1 - b * x1;
            if (b < 0) {
                double Es = -a / (3 * b);
                if (Es > x1 && Es < x2) {
                    double vs = sqrt(2 * Es * OR_QE / m_red) * (a + b * Es);
                    if (vs > best) best = vs;
                }
            }
        }
    }
    return best * 1.0001;
}

static inline double len3(const double v[3]) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

/* MC_MEX_Ionization::newVelocityElecton, LAB form (Interactions.cpp:845-870), with the
 * reference's unnormalised perpendicular basis (i x u, u x (i x u)). */
static void new_vel_electron(double vel[3], double E, const double u[3], double r_pow, double r_phi) {
    double cos_ksi = (2 + E - 2 * pow(1 + E, r_pow)) / E;
    double sin_ksi = sqrt(1 - cos_ksi * cos_ksi);
    double phi = 2 * OR_PI * r_phi;
    double v_mag = sqrt(E * (2 * OR_QE / OR_ME));
    double a[3] = {0 * u[2] - 0 * u[1], 0 * u[0] - 1 * u[2], 1 * u[1] - 0 * u[0]}; /* i x u */
    double b[3] = {u[1] * a[2] - u[2] * a[1], u[2] * a[0] - u[0] * a[2], u[0] * a[1] - u[1] * a[0]};
    double sp = sin(phi), cph = cos(phi);
    for (int d = 0; d < 3; d++) {
        vel[d] = cos_ksi * u[d] + a[d] * sin_ksi * sp + b[d] * sin_ksi * cph;
        vel[d] *= v_mag;
    }
}

/* MC_MEX_Ionization::collide with IONIZE_1 (Interactions.cpp:885-947).  Uniform draws are
 * supplied by the caller in the order the reference consumes rnd(): u_ion, then either
 * (E_ej, pow1, phi1, pow2, phi2) or (cos, eps). */
typedef double (*draw_fn)(void* st);
static void collide(const or_coll_params* cp, const double vel_neu[3], double vel_ele[3], int* ionize,
                    double vel_new[3], double sigma_coll, draw_fn draw, void* st) {
    double m_n = cp->mass_neutral, m_e = cp->mass_electron;
    double m_red = m_n * m_e / (m_n + m_e), sum_mass = m_n + m_e;
    double v_rel[3] = {vel_neu[0] - vel_ele[0], vel_neu[1] - vel_ele[1], vel_neu[2] - vel_ele[2]};
    double v_rel_mag = len3(v_rel);
    double E_rel_J = 0.5 * m_red * v_rel_mag * v_rel_mag;
    double P = or_sigma_ion(cp, E_rel_J / OR_QE) / sigma_coll;
    if (draw(st) <= P) {
        *ionize = 1;
        double vmag = len3(vel_ele);
        double E_inc = vmag * vmag * (OR_ME * 0.5 / OR_QE);
        if (E_inc < cp->E_ion_eV) {
            *ionize = 0;
            return;
        }
        double E_ej = 10.0 * tan(draw(st) * atan((E_inc - cp->E_ion_eV) / (2 * cp->B_inc)));
        double E_sc = E_inc - cp->E_ion_eV - E_ej;
        if (E_sc < 0) E_sc = 0.000001;
        double inv = 1.0 / vmag; /* Vec3::unit divides through 1/l (Vec3.h:110-120, 180-191) */
        double u[3] = {vel_ele[0] * inv, vel_ele[1] * inv, vel_ele[2] * inv};
        double r1 = draw(st), r2 = draw(st);
        new_vel_electron(vel_ele, E_sc, u, r1, r2);
        double r3 = draw(st), r4 = draw(st);
        new_vel_electron(vel_new, E_ej, u, r3, r4);
    } else {
        *ionize = 0;
        double cm[3];
        double inv_sum = 1.0 / sum_mass;
        for (int d = 0; d < 3; d++) cm[d] = (m_n * vel_neu[d] + m_e * vel_ele[d]) * inv_sum;
        double cos_ksi = 2 * draw(st) - 1;
        double sin_ksi = sqrt(1 - cos_ksi * cos_ksi);
        double eps = 2 * OR_PI * draw(st);
        v_rel[0] = v_rel_mag * cos_ksi;
        v_rel[1] = v_rel_mag * sin_ksi * cos(eps);
        v_rel[2] = v_rel_mag * sin_ksi * sin(eps);
        for (int d = 0; d < 3; d++) vel_ele[d] = cm[d] - m_n / sum_mass * v_rel[d];
    }
}
static double mt_draw(void* st) { return or_mt_u01((or_mt*)st); }

/* Philox draw stream for one electron: counter (id_lo, id_hi, step, block) */
typedef struct {
    uint32_t key[2], ctr[4];
    uint32_t buf[4];
    int pos;
} phx_stream;
static void phx_block(phx_stream* s, uint32_t block) {
    s->ctr[3] = block;
    or_philox4x32_10(s->ctr, s->key, s->buf);
    s->pos = 0;
}
/* Collision draws after the candidate test come from blocks 2 and 3 in order:
 *   u_ion, then ionising: E_ej, pow1, phi1, pow2, phi2 ; elastic: cos, eps */
static double phx_draw(void* st) {
    phx_stream* s = (phx_stream*)st;
    if (s->pos >= 4) phx_block(s, s->ctr[3] + 1);
    return or_u01_from_u32(s->buf[s->pos++]);
}

/* Electron-impact collisions against a uniform Maxwellian background (GPU form).
 * Equivalent in expectation to the reference NTC (Interactions.cpp:646-678) when the
 * neutral weight exceeds the electron weight: each electron is a candidate with
 * probability P_null = n_n (sigma v)_max dt and is accepted with sigma v_rel/(sigma v)_max.
 * Candidate test: or_cand_draw(id, step, seed) < or_cand_threshold(P_null).
 * Draw layout per candidate, counter (id_lo, id_hi, step, block):
 *   block 0: a0 unused | a1,a2 Box-Muller (vx,vy) | a3 acceptance
 *   block 1: b0,b1 Box-Muller (vz) | b2,b3 product offset x,y
 *   blocks 2,3: the collide() draws in phx_draw order (at most six)
 *   block 4: word 0 product offset z
 * The ion takes the sampled neutral velocity (vel_splitted_neu, Interactions.cpp:694).
 * Products appear at a uniform point of the parent's cell (the reference places them at a
 * random neutral of the cell, Interactions.cpp:694-695), without velocity rewind. */
long or_mcc_background(const or_grid* g, const or_coll_params* cp, or_particle* ele, uint64_t* ele_id, long* n_ele,
                       long cap_ele, or_particle* ion, uint64_t* ion_id, long* n_ion, long cap_ion, double dt,
                       uint32_t seed_lo, uint32_t seed_hi, uint32_t step, long* n_ionized) {
    double m_n = cp->mass_neutral, m_e = cp->mass_electron;
    double m_red = m_n * m_e / (m_n + m_e);
    double E_precalc_rel_eV = 0.5 * m_red / OR_QE;
    uint32_t cand_max = or_cand_threshold(cp->n_neutral * cp->sigv_max * dt);
    double sig_n = sqrt(OR_KB * cp->T_neutral / m_n);
    const double TWO_PI = 6.283185307179586;
    long n0 = *n_ele, ncoll = 0, nion = 0;
    for (long p = 0; p < n0; p++) {
        if (!(or_cand_draw(ele_id[p], step, seed_lo, seed_hi) < cand_max)) continue;
        phx_stream st;
        st.key[0] = seed_lo;
        st.key[1] = seed_hi;
        st.ctr[0] = (uint32_t)ele_id[p];
        st.ctr[1] = (uint32_t)(ele_id[p] >> 32);
        st.ctr[2] = step;
        phx_block(&st, 0);
        uint32_t a[4] = {st.buf[0], st.buf[1], st.buf[2], st.buf[3]};
        phx_block(&st, 1);
        uint32_t b[4] = {st.buf[0], st.buf[1], st.buf[2], st.buf[3]};
        double r1 = sqrt(-2 * log(or_u01_from_u32(a[1]))), t1 = TWO_PI * or_u01_from_u32(a[2]);
        double r2 = sqrt(-2 * log(or_u01_from_u32(b[0]))), t2 = TWO_PI * or_u01_from_u32(b[1]);
        double vn[3] = {sig_n * r1 * cos(t1), sig_n * r1 * sin(t1), sig_n * r2 * cos(t2)};
        double* ve = ele[p].vel;
        double vr[3] = {vn[0] - ve[0], vn[1] - ve[1], vn[2] - ve[2]};
        double v_rel = len3(vr);
        double E_rel = E_precalc_rel_eV * v_rel * v_rel;
        double sigma = or_sigma_coll(cp, E_rel);
        if (!(or_u01_from_u32(a[3]) * cp->sigv_max < sigma * v_rel)) continue;
        ncoll++;
        phx_block(&st, 2);
        int ionized = 0;
        double vnew[3] = {0, 0, 0};
        collide(cp, vn, ve, &ionized, vnew, sigma, phx_draw, &st);
        if (!ionized) continue;
        nion++;
        double lc[3];
        xtol(g, ele[p].pos, lc);
        double pos[3];
        phx_block(&st, 4);
        double uo[3] = {or_u01_from_u32(b[2]), or_u01_from_u32(b[3]), or_u01_from_u32(st.buf[0])};
        for (int d = 0; d < 3; d++) pos[d] = g->x0[d] + ((double)(int)lc[d] + uo[d]) * g->dx[d];
        uint64_t pid = ele_id[p];
        if (*n_ele < cap_ele) {
            or_particle* q = &ele[*n_ele];
            for (int d = 0; d < 3; d++) {
                q->pos[d] = pos[d];
                q->vel[d] = vnew[d];
            }
            q->w = ele[p].w;
            ele_id[*n_ele] = or_child_id(pid, step, 1);
            (*n_ele)++;
        }
        if (*n_ion < cap_ion) {
            or_particle* q = &ion[*n_ion];
            for (int d = 0; d < 3; d++) {
                q->pos[d] = pos[d];
                q->vel[d] = vn[d];
            }
            q->w = ele[p].w;
            ion_id[*n_ion] = or_child_id(pid, step, 2);
            (*n_ion)++;
        }
    }
    if (n_ionized) *n_ionized = nion;
    return ncoll;
}

/* ---- cell lists as Species::sortIndexes (Species.cpp:905-915) ---- */
typedef struct {
    long* idx;
    long n, cap;
} ilist;
static void il_push(ilist* l, long v) {
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 8;
        l->idx = (long*)realloc(l->idx, sizeof(long) * l->cap);
    }
    l->idx[l->n++] = v;
}
static int xtoc(const or_grid* g, const double x[3]) {
    double lc[3];
    xtol(g, x, lc);
    return ((int)lc[2] * (g->nj - 1) + (int)lc[1]) * (g->ni - 1) + (int)lc[0];
}
static ilist* sort_indexes(const or_grid* g, const or_particle* p, long n) {
    long nc = (long)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    ilist* cells = (ilist*)calloc(nc, sizeof(ilist));
    for (long q = 0; q < n; q++) il_push(&cells[xtoc(g, p[q].pos)], q);
    return cells;
}
static void free_cells(ilist* c, long nc) {
    for (long i = 0; i < nc; i++) free(c[i].idx);
    free(c);
}

/* MC_MEX_Ionization::apply_vector_indexes (Interactions.cpp:600-762), including its quirks:
 * the differential electron of an electron split gets weight 0 (line 709 reads the weight
 * after line 707 overwrote it); a deleted neutral is overwritten by the last neutral and the
 * tail is erased after the cell loop (lines 721, 757-758). */
long or_ntc_ionize_ref(const or_grid* g, const or_coll_params* cp, or_mt* r, or_particle* neu, long* n_neu,
                       long cap_neu, or_particle* ion, long* n_ion, long cap_ion, or_particle* ele, long* n_ele,
                       long cap_ele, double dt, double* wsv_max) {
    double m_n = cp->mass_neutral, m_e = cp->mass_electron;
    double m_red = m_n * m_e / (m_n + m_e);
    double E_precalc_rel_eV = 0.5 * m_red / OR_QE;
    double inv_dv = 1 / (g->dx[0] * g->dx[1] * g->dx[2]);
    long nc = (long)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    ilist* Nc = sort_indexes(g, neu, *n_neu);
    ilist* Ec = sort_indexes(g, ele, *n_ele);
    double wsv_tmp = 0;
    long n_coll = 0, to_delete = 0;
    for (long c = 0; c < nc; c++) {
        ilist* ie = &Ec[c];
        int ne = (int)ie->n;
        if (ne <= 0) continue;
        ilist* in = &Nc[c];
        int nn = (int)in->n;
        if (nn <= 0) continue;
        double frac = (double)(nn * ne) * *wsv_max * dt * inv_dv;
        int n_groups = (int)(frac + 0.5);
        if (n_groups > nn) n_groups = nn - 1;
        for (int gi = 0; gi < n_groups; gi++) {
            int ns = (int)mt_range(r, 0, nn);
            long p_neu = in->idx[ns];
            int es = (int)mt_range(r, 0, ne);
            long p_ele = ie->idx[es];
            double vr[3] = {neu[p_neu].vel[0] - ele[p_ele].vel[0], neu[p_neu].vel[1] - ele[p_ele].vel[1],
                            neu[p_neu].vel[2] - ele[p_ele].vel[2]};
            double v_rel = len3(vr);
            double E_rel = E_precalc_rel_eV * v_rel * v_rel;
            double sigma = or_sigma_coll(cp, E_rel);
            double Wg = neu[p_neu].w, Wl = ele[p_ele].w;
            if (Wg < Wl) {
                double t = Wg;
                Wg = Wl;
                Wl = t;
            }
            double wsv = Wg * sigma * v_rel;
            if (wsv > wsv_tmp) wsv_tmp = wsv;
            double P = wsv / *wsv_max;
            if (!(or_mt_u01(r) < P)) continue;
            n_coll++;
            or_particle* e = &ele[p_ele];
            or_particle* nu = &neu[p_neu];
            int ionised = 0;
            double vnew[3] = {0, 0, 0};
            if (nu->w > e->w) {
                nu->w -= e->w;
                double vsplit[3] = {nu->vel[0], nu->vel[1], nu->vel[2]};
                collide(cp, vsplit, e->vel, &ionised, vnew, sigma, mt_draw, r);
                if (ionised) {
                    if (*n_ion < cap_ion) ion[(*n_ion)++] = (or_particle){{nu->pos[0], nu->pos[1], nu->pos[2]},
                                                                        {vsplit[0], vsplit[1], vsplit[2]}, Wl};
                    if (*n_ele < cap_ele) ele[(*n_ele)++] = (or_particle){{nu->pos[0], nu->pos[1], nu->pos[2]},
                                                                        {vnew[0], vnew[1], vnew[2]}, Wl};
                } else {
                    if (*n_neu < cap_neu) {
                        neu[*n_neu] = (or_particle){{nu->pos[0], nu->pos[1], nu->pos[2]},
                                                    {nu->vel[0], nu->vel[1], nu->vel[2]}, e->w};
                        il_push(in, *n_neu);
                        (*n_neu)++;
                        nn++;
                    }
                }
            } else if (nu->w < e->w) {
                e->w = nu->w;
                if (*n_ele < cap_ele) {
                    ele[*n_ele] = (or_particle){{e->pos[0], e->pos[1], e->pos[2]},
                                                {e->vel[0], e->vel[1], e->vel[2]}, e->w - nu->w};
                    il_push(ie, *n_ele);
                    (*n_ele)++;
                }
                e = &ele[p_ele];
                collide(cp, nu->vel, e->vel, &ionised, vnew, sigma, mt_draw, r);
                if (ionised) {
                    if (*n_ion < cap_ion) ion[(*n_ion)++] = (or_particle){{nu->pos[0], nu->pos[1], nu->pos[2]},
                                                                        {nu->vel[0], nu->vel[1], nu->vel[2]}, Wl};
                    if (*n_ele < cap_ele) ele[(*n_ele)++] = (or_particle){{nu->pos[0], nu->pos[1], nu->pos[2]},
                                                                        {vnew[0], vnew[1], vnew[2]}, Wl};
                    nn--;
                    in->idx[ns] = in->idx[nn];
                    neu[p_neu] = neu[*n_neu - 1];
                    to_delete++;
                }
            }
        }
    }
    if (n_coll) {
        *wsv_max = wsv_tmp;
        if (to_delete) *n_neu -= to_delete;
    }
    free_cells(Nc, nc);
    free_cells(Ec, nc);
    return n_coll;
}

/* Species::addParticle (Species.cpp:420-434): reject NaN / out of bounds / in object, then
 * rewind v by half a (global) step with the gathered E. */
static int add_particle(const or_grid* g, or_particle* p, long* n, long cap, const double pos[3], const double vel[3],
                        double w, const double* ef, double charge, double mass, double dt) {
    for (int d = 0; d < 3; d++)
        if (isnan(pos[d]) || isnan(vel[d])) return 0;
    for (int d = 0; d < 3; d++)
        if (pos[d] < g->x0[d] || pos[d] >= g->xm[d]) return 0;
    if (in_object(g, pos)) return 0;
    double lc[3], e[3] = {0, 0, 0};
    xtol(g, pos, lc);
    if (ef) or_gather3_ref(g, ef, lc, e);
    if (*n >= cap) return 0;
    or_particle* q = &p[(*n)++];
    for (int d = 0; d < 3; d++) {
        q->pos[d] = pos[d];
        q->vel[d] = vel[d] - charge / mass * e[d] * (0.5 * dt);
    }
    q->w = w;
    return 1;
}

/* Species::merge + sortVelocitiesInCell (Species.cpp:981-1145). */
long or_merge_ref(const or_grid* g, or_mt* r, or_particle* p, long n, long cap, const double* ef, double charge,
                  double mass, double dt_global, int min_count) {
    if (n == 0) return 0;
    long nc = (long)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    ilist* cells = sort_indexes(g, p, n);
    const int NG = 15;
    ilist* bins = (ilist*)calloc(NG * NG * NG, sizeof(ilist));
    long np = n;
    for (long c = 0; c < nc; c++) {
        ilist* cl = &cells[c];
        if (cl->n < min_count) continue;
        /* velocity range; starts from particles[0] of the species (Species.cpp:985) */
        double vmin[3] = {p[0].vel[0], p[0].vel[1], p[0].vel[2]}, vmax[3] = {p[0].vel[0], p[0].vel[1], p[0].vel[2]};
        for (long q = 0; q < cl->n; q++) {
            const double* v = p[cl->idx[q]].vel;
            for (int d = 0; d < 3; d++) {
                if (v[d] < vmin[d]) vmin[d] = v[d];
                else if (v[d] > vmax[d]) vmax[d] = v[d];
            }
        }
        for (int d = 0; d < 3; d++) vmax[d] *= vmax[d] > 0 ? 1.001 : 0.999;
        double dv[3];
        for (int d = 0; d < 3; d++) dv[d] = (vmax[d] - vmin[d]) / 15.0;
        for (int b = 0; b < NG * NG * NG; b++) bins[b].n = 0;
        for (long q = 0; q < cl->n; q++) {
            const double* v = p[cl->idx[q]].vel;
            int bi[3];
            for (int d = 0; d < 3; d++) {
                bi[d] = (int)((v[d] - vmin[d]) / dv[d]);
                if (bi[d] < 0) bi[d] = 0; /* out-of-range indices are undefined in the reference */
                if (bi[d] > NG - 1) bi[d] = NG - 1;
            }
            il_push(&bins[(bi[0] * NG + bi[1]) * NG + bi[2]], cl->idx[q]);
        }
        for (int b = 0; b < NG * NG * NG; b++) {
            ilist* vb = &bins[b];
            if (vb->n <= 2) continue;
            double W = 0, M[3] = {0, 0, 0}, E[3] = {0, 0, 0};
            for (long q = 0; q < vb->n; q++) {
                or_particle* pp = &p[vb->idx[q]];
                W += pp->w;
                for (int d = 0; d < 3; d++) M[d] += pp->w * pp->vel[d];
                for (int d = 0; d < 3; d++) E[d] += pp->w * (pp->vel[d] * pp->vel[d]);
                pp->w = 0;
            }
            double wa = W * 0.5, wb = W * 0.5;
            double invW = 1.0 / W; /* Vec3::operator/= multiplies by 1/val (Vec3.h:212-222) */
            for (int d = 0; d < 3; d++) M[d] *= invW;
            for (int d = 0; d < 3; d++) E[d] *= invW;
            for (int d = 0; d < 3; d++) E[d] -= M[d] * M[d];
            for (int d = 0; d < 3; d++)
                if (E[d] < 0) {
                    if (E[d] < -10e-5) break;
                    E[d] = 0;
                }
            double sq[3] = {sqrt(E[0]), sqrt(E[1]), sqrt(E[2])};
            double va[3], vb3[3];
            for (int d = 0; d < 3; d++) {
                va[d] = M[d] + sq[d];
                vb3[d] = M[d] - sq[d];
            }
            int cs = (int)vb->n;
            long pa = vb->idx[(int)mt_range(r, 0, cs)];
            long pb = vb->idx[(int)mt_range(r, 0, cs)];
            while (pb == pa) pb = vb->idx[(int)mt_range(r, 0, cs)];
            double posa[3] = {p[pa].pos[0], p[pa].pos[1], p[pa].pos[2]};
            double posb[3] = {p[pb].pos[0], p[pb].pos[1], p[pb].pos[2]};
            add_particle(g, p, &np, cap, posa, va, wa, ef, charge, mass, dt_global);
            add_particle(g, p, &np, cap, posb, vb3, wb, ef, charge, mass, dt_global);
        }
    }
    for (long q = 0; q < np; q++)
        if (p[q].w == 0) {
            p[q] = p[np - 1];
            np--;
            q--;
        }
    for (int b = 0; b < NG * NG * NG; b++) free(bins[b].idx);
    free(bins);
    free_cells(cells, nc);
    return np;
}

static int vel_bin_f(float v, float vmin, float dv) {
    if (!(dv > 0.f)) return 0;
    int b = (int)((v - vmin) / dv);
    return b < 0 ? 0 : (b > 14 ? 14 : b);
}
typedef struct {
    uint64_t key;
    long idx;
} mkey;
static int cmp_mkey(const void* a, const void* b) {
    uint64_t x = ((const mkey*)a)->key, y = ((const mkey*)b)->key;
    return (x > y) - (x < y);
}
long or_merge_gpuform(const or_grid* g, or_particle* p, uint64_t* ids, const int32_t* cells, long n, long cap,
                      const double* ef, double charge, double mass, double dt_global, int min_count,
                      uint32_t seed_lo, uint32_t seed_hi, uint32_t step) {
    long nc = (long)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    ilist* cl = (ilist*)calloc(nc, sizeof(ilist));
    for (long q = 0; q < n; q++) il_push(&cl[cells ? cells[q] : xtoc(g, p[q].pos)], q);
    long np = n;
    uint32_t key[2] = {seed_lo, seed_hi};
    for (long c = 0; c < nc; c++) {
        long m = cl[c].n;
        if (m < min_count) continue;
        if (m > 1024) m = 1024; /* the device handles 1024 particles per cell and flags the rest */
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (long q = 0; q < m; q++)
            for (int d = 0; d < 3; d++) {
                float v = (float)p[cl[c].idx[q]].vel[d];
                lo[d] = fminf(lo[d], v);
                hi[d] = fmaxf(hi[d], v);
            }
        float dv[3];
        for (int d = 0; d < 3; d++) {
            hi[d] = hi[d] > 0.f ? hi[d] * 1.001f : hi[d] * 0.999f;
            dv[d] = (hi[d] - lo[d]) / 15.0f;
        }
        mkey* keys = (mkey*)malloc(sizeof(mkey) * m);
        for (long q = 0; q < m; q++) {
            long pi = cl[c].idx[q];
            int b = (vel_bin_f((float)p[pi].vel[0], lo[0], dv[0]) * 15 + vel_bin_f((float)p[pi].vel[1], lo[1], dv[1])) *
                        15 + vel_bin_f((float)p[pi].vel[2], lo[2], dv[2]);
            uint32_t ctr[4] = {(uint32_t)ids[pi], (uint32_t)(ids[pi] >> 32), step, 0x4D455247u}, out[4];
            or_philox4x32_10(ctr, key, out);
            uint64_t hh = (((uint64_t)out[1] << 32) | out[0]) & ((1ull << 42) - 1);
            keys[q].key = ((uint64_t)b << 52) | (hh << 10) | (uint64_t)q;
            keys[q].idx = pi;
        }
        qsort(keys, m, sizeof(mkey), cmp_mkey);
        for (long q = 0; q < m;) {
            long e = q + 1;
            while (e < m && (keys[e].key >> 52) == (keys[q].key >> 52)) e++;
            if (e - q > 2) {
                double W = 0, M[3] = {0, 0, 0}, E[3] = {0, 0, 0};
                for (long r = q; r < e; r++) {
                    or_particle* pp = &p[keys[r].idx];
                    double w = (float)pp->w;
                    double v3[3] = {(float)pp->vel[0], (float)pp->vel[1], (float)pp->vel[2]};
                    W += w;
                    for (int d = 0; d < 3; d++) M[d] += w * v3[d];
                    for (int d = 0; d < 3; d++) E[d] += w * (v3[d] * v3[d]);
                }
                double inv = 1.0 / W;
                for (int d = 0; d < 3; d++) {
                    M[d] *= inv;
                    E[d] = E[d] * inv - M[d] * M[d];
                }
                for (int d = 0; d < 3; d++)
                    if (E[d] < 0) {
                        if (E[d] < -10e-5) break;
                        E[d] = 0;
                    }
                double sq[3] = {sqrt(E[0]), sqrt(E[1]), sqrt(E[2])};
                for (int side = 0; side < 2; side++) {
                    long src = keys[q + side].idx;
                    double sgn = side == 0 ? 1.0 : -1.0;
                    double v[3] = {(float)(M[0] + sgn * sq[0]), (float)(M[1] + sgn * sq[1]), (float)(M[2] + sgn * sq[2])};
                    if (isnan(v[0]) || isnan(v[1]) || isnan(v[2]) || np >= cap) continue;
                    double lc[3], e3[3] = {0, 0, 0};
                    xtol(g, p[src].pos, lc);
                    if (ef) or_gather3_ref(g, ef, lc, e3);
                    or_particle* o = &p[np];
                    for (int d = 0; d < 3; d++) {
                        o->pos[d] = p[src].pos[d];
                        o->vel[d] = v[d] - charge / mass * 0.5 * dt_global * e3[d];
                    }
                    o->w = (float)(W * 0.5);
                    ids[np] = or_child_id(ids[src], step, 3);
                    np++;
                }
                for (long r = q; r < e; r++) p[keys[r].idx].w = 0;
            }
            q = e;
        }
        free(keys);
    }
    /* remove merged members keeping the order of the rest */
    long k = 0;
    for (long q = 0; q < np; q++)
        if (p[q].w != 0) {
            p[k] = p[q];
            ids[k] = ids[q];
            k++;
        }
    free_cells(cl, nc);
    return k;
}

/* Species::sampleVth / sampleV3th (Species.cpp:855-869) */
static double sample_vth(or_mt* r, double T, double mass) {
    double v_th = sqrt(2 * OR_KB * T / mass);
    double v1 = v_th * (or_mt_u01(r) + or_mt_u01(r) + or_mt_u01(r) - 1.5);
    double v2 = v_th * (or_mt_u01(r) + or_mt_u01(r) + or_mt_u01(r) - 1.5);
    double v3 = v_th * (or_mt_u01(r) + or_mt_u01(r) + or_mt_u01(r) - 1.5);
    return sqrt(v1 * v1 + v2 * v2 + v3 * v3);
}
long or_load_box_thermal_ref(const or_grid* g, or_mt* r, or_particle* p, long cap, const double* x0,
                             const double* sides, double num_den, double T, double mpw0, double mass, double charge,
                             const double* ef, double dt) {
    double box_vol = sides[0] * sides[1] * sides[2];
    double num_micro = num_den * box_vol;
    long num_macro = (long)(num_micro / mpw0);
    double xmin[3], xmax[3];
    for (int d = 0; d < 3; d++) {
        xmin[d] = x0[d] - sides[d] / 2;
        xmax[d] = x0[d] + sides[d] / 2;
    }
    long n = 0;
    for (long q = 0; q < num_macro; q++) {
        double pos[3];
        pos[0] = mt_range(r, xmin[0], xmax[0]);
        pos[1] = mt_range(r, xmin[1], xmax[1]);
        pos[2] = mt_range(r, xmin[2], xmax[2]);
        double v_th = sample_vth(r, T, mass);
        double theta = 2 * OR_PI * or_mt_u01(r);
        double rr = -1.0 + 2 * or_mt_u01(r);
        double a = sqrt(1 - rr * rr);
        double vel[3] = {v_th * rr, v_th * (cos(theta) * a), v_th * (sin(theta) * a)};
        add_particle(g, p, &n, cap, pos, vel, mpw0, ef, charge, mass, dt);
    }
    return n;
}

void or_sample_moments_ref(const or_grid* g, const or_particle* p, long n, double* mom) {
    long nv = (long)g->ni * g->nj * g->nk;
    for (long q = 0; q < n; q++) {
        double lc[3];
        xtol(g, p[q].pos, lc);
        double w = p[q].w;
        or_scatter_ref(g, mom, lc, w);
        for (int d = 0; d < 3; d++) or_scatter_ref(g, mom + (1 + d) * nv, lc, w * p[q].vel[d]);
        for (int d = 0; d < 3; d++) or_scatter_ref(g, mom + (4 + d) * nv, lc, w * p[q].vel[d] * p[q].vel[d]);
    }
}
void or_gas_properties_ref(const or_grid* g, const double* mom, double mass, double* vel, double* T) {
    long nv = (long)g->ni * g->nj * g->nk;
    for (long n = 0; n < nv; n++) {
        double cnt = mom[n];
        for (int d = 0; d < 3; d++) vel[3 * n + d] = cnt != 0 ? mom[(1 + d) * nv + n] * (1.0 / cnt) : 0;
        if (cnt <= 0) {
            T[n] = 0;
            continue;
        }
        double uu = mom[4 * nv + n] / cnt - vel[3 * n] * vel[3 * n];
        double vv = mom[5 * nv + n] / cnt - vel[3 * n + 1] * vel[3 * n + 1];
        double ww = mom[6 * nv + n] / cnt - vel[3 * n + 2] * vel[3 * n + 2];
        T[n] = mass / (2 * OR_KB) * (uu + vv + ww);
    }
}

void or_sums(const or_particle* p, long n, double mass, double* count, double mom[3], double* ke) {
    double c = 0, m[3] = {0, 0, 0}, k = 0;
    for (long q = 0; q < n; q++) {
        c += p[q].w;
        for (int d = 0; d < 3; d++) m[d] += p[q].w * p[q].vel[d];
        k += p[q].w * (p[q].vel[0] * p[q].vel[0] + p[q].vel[1] * p[q].vel[1] + p[q].vel[2] * p[q].vel[2]);
    }
    *count = c;
    for (int d = 0; d < 3; d++) mom[d] = m[d] * mass;
    *ke = k * mass * 0.5;
}

/* ---- DSMC_MEX (Interactions.cpp:143-284) ---- */
void or_dsmc_params_init(or_dsmc_params* q, const or_grid* g, double mass1, double mass2, double mpw0) {
    q->mass1 = mass1;
    q->mass2 = mass2;
    q->mpw0 = mpw0;
    q->dv = g->dx[0] * g->dx[1] * g->dx[2];
    double m_red = mass1 * mass2 / (mass1 + mass2);
    q->c[0] = 4.07e-10; /* Bird's VHS reference diameter and viscosity index, at 273.15 K */
    q->c[1] = 0.77;
    q->c[2] = 2 * OR_KB * 273.15 / m_red;
    q->c[3] = tgamma(2.5 - q->c[1]);
}
double or_dsmc_sigma(const or_dsmc_params* q, double v_rel) {
    return OR_PI * q->c[0] * q->c[0] * pow(q->c[2] / (v_rel * v_rel), q->c[1] - 0.5) / q->c[3];
}
/* DSMC_MEX::collide (Interactions.cpp:264-284): isotropic scattering in the centre-of-mass frame */
static void dsmc_collide_ref(const or_dsmc_params* q, or_mt* r, double v1[3], double v2[3]) {
    double sum_mass = q->mass1 + q->mass2, inv = 1.0 / sum_mass;
    double cm[3], vr[3];
    for (int d = 0; d < 3; d++) cm[d] = (v1[d] * q->mass1 + v2[d] * q->mass2) * inv;
    for (int d = 0; d < 3; d++) vr[d] = v1[d] - v2[d];
    double mag = len3(vr);
    double cos_ksi = 2 * or_mt_u01(r) - 1;
    double sin_ksi = sqrt(1 - cos_ksi * cos_ksi);
    double eps = 2 * OR_PI * or_mt_u01(r);
    vr[0] = mag * cos_ksi;
    vr[1] = mag * sin_ksi * cos(eps);
    vr[2] = mag * sin_ksi * sin(eps);
    double f2 = q->mass2 / sum_mass, f1 = q->mass1 / sum_mass;
    for (int d = 0; d < 3; d++) {
        v1[d] = cm[d] + vr[d] * f2;
        v2[d] = cm[d] - vr[d] * f1;
    }
}
long or_dsmc_ref(const or_grid* g, const or_dsmc_params* q, or_mt* r, or_particle* p1, long n1, or_particle* p2,
                 long n2, double dt, double* svmax, long* pairs) {
    int one = p2 == NULL;
    long nc = (long)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    ilist* C1 = sort_indexes(g, p1, n1);
    ilist* C2 = one ? C1 : sort_indexes(g, p2, n2);
    or_particle* q2 = one ? p1 : p2;
    double sv_tmp = 0;
    long n_coll = 0, n_pairs = 0;
    for (long c = 0; c < nc; c++) {
        int a = (int)C1[c].n, b = (int)C2[c].n;
        if (one ? a < 2 : (a < 1 || b < 1)) continue;
        double frac = 0.5 * a * b * q->mpw0 * *svmax * dt / q->dv;
        int n_groups = (int)(frac + 0.5);
        for (int gi = 0; gi < n_groups; gi++) {
            int i1 = (int)(or_mt_u01(r) * a);
            int i2 = (int)(or_mt_u01(r) * b);
            while (one && i1 == i2) i2 = (int)(or_mt_u01(r) * b);
            double* v1 = p1[C1[c].idx[i1]].vel;
            double* v2 = q2[C2[c].idx[i2]].vel;
            double vr[3] = {v1[0] - v2[0], v1[1] - v2[1], v1[2] - v2[2]};
            double v_rel = len3(vr);
            double sv = or_dsmc_sigma(q, v_rel) * v_rel;
            if (sv > sv_tmp) sv_tmp = sv;
            double P = sv / *svmax;
            n_pairs++;
            if (P > or_mt_u01(r)) {
                n_coll++;
                dsmc_collide_ref(q, r, v1, v2);
            }
        }
    }
    if (n_coll) *svmax = sv_tmp;
    if (pairs) *pairs = n_pairs;
    free_cells(C1, nc);
    if (!one) free_cells(C2, nc);
    return n_coll;
}
long or_dsmc_gpuform(const or_dsmc_params* q, double* vel1, const int32_t* cnt1, double* vel2, const int32_t* cnt2,
                     long nc, double dt, double svmax, uint32_t seed_lo, uint32_t seed_hi, uint32_t call,
                     uint32_t tag, long* pairs, double* svmax_step) {
    int one = vel2 == NULL;
    const uint32_t key[2] = {seed_lo, seed_hi};
    /* sigma(g) g = pi d^2 (c2/g^2)^(omega-1/2) / Gamma * g = K (g^2)^(1-omega); the kernel's
     * constants are FP32 roundings of the FP64 parameters */
    double K = (float)(OR_PI * q->c[0] * q->c[0] * pow(q->c[2], q->c[1] - 0.5) / q->c[3]);
    double ex = (float)(1.0 - q->c[1]);
    double f1 = (float)(q->mass1 / (q->mass1 + q->mass2)), f2 = (float)(q->mass2 / (q->mass1 + q->mass2));
    double half_coef = 0.5 * q->mpw0 * dt / q->dv;
    long s1 = 0, s2 = 0, n_coll = 0, n_pairs = 0;
    double mx = 0;
    for (long c = 0; c < nc; c++) {
        int a = cnt1[c], b = one ? a : cnt2[c];
        double* w1 = vel1 + 3 * s1;
        double* w2 = one ? w1 : vel2 + 3 * s2;
        s1 += a;
        if (!one) s2 += b;
        if (one ? a < 2 : (a < 1 || b < 1)) continue;
        double frac = (double)a * (double)b * (half_coef * svmax);
        int n_groups = (int)(frac + 0.5);
        for (int gi = 0; gi < n_groups; gi++) {
            uint32_t ctr[4] = {(uint32_t)c, call, tag, (uint32_t)gi}, rr[4];
            or_philox4x32_10(ctr, key, rr);
            uint32_t i1 = (uint32_t)(((uint64_t)rr[0] * (uint32_t)a) >> 32);
            uint32_t i2 = (uint32_t)(((uint64_t)rr[1] * (uint32_t)(one ? a - 1 : b)) >> 32);
            if (one && i2 >= i1) i2++;
            double* v1 = w1 + 3 * i1;
            double* v2 = w2 + 3 * i2;
            double d[3] = {v1[0] - v2[0], v1[1] - v2[1], v1[2] - v2[2]};
            double g2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            double sv = K * pow(g2, ex);
            if (sv > mx) mx = sv;
            n_pairs++;
            if (!(sv > or_u01_from_u32(rr[2]) * svmax)) continue;
            n_coll++;
            uint32_t low27 = (rr[0] & 511u) | ((rr[1] & 511u) << 9) | ((rr[2] & 511u) << 18);
            double ck = 2 * or_u01_from_u32(rr[3]) - 1;
            double sk = sqrt(fmax(1 - ck * ck, 0.0));
            double eps = 2 * 3.14159265358979323846 * (((double)low27 + 0.5) / 134217728.0);
            double gm = sqrt(g2);
            double vr[3] = {gm * ck, gm * sk * cos(eps), gm * sk * sin(eps)};
            for (int k = 0; k < 3; k++) {
                double cm = f1 * v1[k] + f2 * v2[k];
                v1[k] = cm + f2 * vr[k];
                v2[k] = cm - f1 * vr[k];
            }
        }
    }
    if (pairs) *pairs = n_pairs;
    if (svmax_step) *svmax_step = mx;
    return n_coll;
}

/* ---- object interaction of non-electron species (Species.cpp:45-256) ---- */
/* Rectangle::lineIntersect (Object.cpp:239-302) */
static void box_line_intersect(const or_grid* g, int b, const double x1[3], const double x2[3], double* t_entry,
                               double xi[3], double n[3]) {
    double tmin[3], tmax[3], A[3];
    int ps[3] = {0, 1, 2};
    for (int d = 0; d < 3; d++) A[d] = x2[d] - x1[d];
    for (int d = 0; d < 3; d++) {
        tmin[d] = (g->box_c[b][d] - g->box_half[b][d] - x1[d]) / A[d];
        tmax[d] = (g->box_c[b][d] + g->box_half[b][d] - x1[d]) / A[d];
    }
    for (int d = 0; d < 3; d++)
        if (tmin[d] > tmax[d]) {
            double t = tmin[d];
            tmin[d] = tmax[d];
            tmax[d] = t;
            ps[d] += 3;
        }
    double te = tmin[0];
    int j = 0, k = 0, t = 0;
    for (int i = 0; i < 2; i++) {
        if (te < tmin[i + 1]) {
            te = tmin[i + 1];
            j = i + 1;
            k = 0;
        } else if (fabs(te - tmin[i + 1]) < 1e-6) {
            k++;
            t = i + 1;
        }
    }
    n[0] = n[1] = n[2] = 0;
    n[ps[j] % 3] += ps[j] < 3 ? -1.0 : 1.0;
    if (k != 0) {
        if (k < 2) {
            n[ps[t] % 3] += ps[t] < 3 ? -1.0 : 1.0;
        } else {
            n[ps[2] % 3] += ps[2] < 3 ? -1.0 : 1.0;
            n[ps[1] % 3] += ps[1] < 3 ? -1.0 : 1.0;
        }
        double inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int d = 0; d < 3; d++) n[d] *= inv;
    }
    for (int d = 0; d < 3; d++) xi[d] = x1[d] + (x2[d] - x1[d]) * te;
    *t_entry = te;
}
typedef double (*draw_fn)(void*);
static double draw_mt(void* r) { return or_mt_u01((or_mt*)r); }
typedef struct {
    uint32_t ctr[4], key[2], buf[4];
    int pos;
} obj_stream;
static double draw_obj(void* s_) {
    obj_stream* s = (obj_stream*)s_;
    if (s->pos == 4) {
        or_philox4x32_10(s->ctr, s->key, s->buf);
        s->ctr[3]++;
        s->pos = 0;
    }
    return or_u01_from_u32(s->buf[s->pos++]);
}
/* Species::sampleReflectedVelocity (Species.cpp:835-853) with sampleVth(300) (855-861) */
static void reflect_vel(double mass, double v_mag1, const double n[3], draw_fn draw, void* r, double out[3]) {
    double v_th0 = sqrt(2 * OR_KB * 300.0 / mass), s3[3];
    for (int d = 0; d < 3; d++) {
        double u1 = draw(r), u2 = draw(r), u3 = draw(r);
        s3[d] = v_th0 * (u1 + u2 + u3 - 1.5);
    }
    double v_th = sqrt(s3[0] * s3[0] + s3[1] * s3[1] + s3[2] * s3[2]);
    double v_mag2 = v_mag1 + 1.0 * (v_th - v_mag1);
    double sin_theta = draw(r);
    double cos_theta = sqrt(1 - sin_theta * sin_theta);
    double psi = 2 * OR_PI * draw(r);
    double t1[3];
    if (n[0] * 1 + n[1] * 0 + n[2] * 0 != 0) {
        t1[0] = n[1] * 0 - n[2] * 0;
        t1[1] = n[2] * 1 - n[0] * 0;
        t1[2] = n[0] * 0 - n[1] * 1;
    } else {
        t1[0] = n[1] * 0 - n[2] * 1;
        t1[1] = n[2] * 0 - n[0] * 0;
        t1[2] = n[0] * 1 - n[1] * 0;
    }
    double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    double a = sin_theta * cos(psi), b = sin(psi);
    for (int d = 0; d < 3; d++) out[d] = (t1[d] * a + t2[d] * b + n[d] * cos_theta) * v_mag2;
}
static int in_bounds(const or_grid* g, const double x[3]) {
    for (int d = 0; d < 3; d++)
        if (x[d] < g->x0[d] || x[d] >= g->xm[d]) return 0;
    return 1;
}
/* what an impact at xi leaves behind for an ion (Species.cpp:225-245); created ids (GPU form
 * only) follow the device's obj_child_id */
static uint64_t obj_child_id(uint64_t parent, uint32_t step, uint32_t k) {
    return or_mix64(or_child_id(parent, step, 3) + (uint64_t)(k + 1) * 0xD1B54A32D192ED03ull);
}
static void ion_impact(const or_grid* g, const or_obj_species* t, double w, double vmag, double mass, const double xi[3],
                       const double n[3], draw_fn draw, void* r, int with_ids, uint64_t id, uint32_t step,
                       long* created) {
    int m = (int)(w / t->neu_mpw0 + draw(r));
    for (int q = 0; q < m; q++) {
        double vn[3];
        reflect_vel(mass, vmag, n, draw, r, vn);
        long before = *t->n_neu;
        add_particle(g, t->neu, t->n_neu, t->cap_neu, xi, vn, t->neu_mpw0, t->ef, t->neu_qm, 1.0, t->dt_global);
        if (*t->n_neu > before) {
            if (with_ids) t->neu_ids[before] = obj_child_id(id, step, (uint32_t)q);
            created[0]++;
        }
    }
    if (t->sputtering) {
        double yield = vmag > 5e3 ? 0.1 : 0;
        int ms = (int)(yield * w / t->spu_mpw0 + draw(r));
        for (int q = 0; q < ms; q++) {
            double vn[3];
            reflect_vel(mass, vmag, n, draw, r, vn);
            long before = *t->n_spu;
            add_particle(g, t->spu, t->n_spu, t->cap_spu, xi, vn, t->spu_mpw0, t->ef, t->spu_qm, 1.0, t->dt_global);
            if (*t->n_spu > before) {
                if (with_ids) t->spu_ids[before] = obj_child_id(id, step, 0x10000000u + (uint32_t)q);
                created[1]++;
            }
        }
    }
}
long or_push_nonelectron_ref(const or_grid* g, or_mt* r, or_particle* p, long n, const double* ef, double dt,
                             double charge, double mass, const or_obj_species* t, long created[2]) {
    double factor = dt * charge / mass;
    long np = n;
    created[0] = created[1] = 0;
    for (long q = 0; q < np; q++) {
        or_particle* part = &p[q];
        double lc[3], e[3];
        xtol(g, part->pos, lc);
        or_gather3_ref(g, ef, lc, e);
        for (int d = 0; d < 3; d++) part->vel[d] += e[d] * factor;
        double t_rem = 1;
        int nb = 0, removed = 0;
        while (t_rem > 0) {
            if (++nb > 20) {
                removed = 1;
                break;
            }
            double pos_old[3] = {part->pos[0], part->pos[1], part->pos[2]};
            for (int d = 0; d < 3; d++) part->pos[d] += part->vel[d] * t_rem * dt;
            int obj = in_object(g, part->pos);
            if (!in_bounds(g, part->pos)) {
                removed = 1;
                break;
            } else if (obj) {
                double tp, xi[3], nrm[3];
                box_line_intersect(g, obj - 1, pos_old, part->pos, &tp, xi, nrm);
                for (int d = 0; d < 3; d++) part->pos[d] = xi[d];
                double vmag = len3(part->vel);
                if (charge == 0) {
                    reflect_vel(mass, len3(part->vel), nrm, draw_mt, r, part->vel);
                } else {
                    ion_impact(g, t, part->w, vmag, mass, xi, nrm, draw_mt, r, 0, 0, 0, created);
                    removed = 1;
                    break;
                }
                t_rem *= (1 - tp);
                continue;
            }
            t_rem = 0;
        }
        if (removed) {
            p[q] = p[np - 1];
            np--;
            q--;
        }
    }
    return np;
}
long or_push_nonelectron_gpuform(const or_grid* g, or_particle* p, uint64_t* ids, long n, const double* ef, double dt,
                                 double charge, double mass, const or_obj_species* t, uint32_t seed_lo,
                                 uint32_t seed_hi, uint32_t step, long stats[4]) {
    double factor = dt * charge / mass;
    long np = n;
    for (int k = 0; k < 4; k++) stats[k] = 0;
    for (long q = 0; q < np; q++) {
        or_particle* part = &p[q];
        double lc[3], e[3];
        xtol(g, part->pos, lc);
        or_gather3_ref(g, ef, lc, e);
        for (int d = 0; d < 3; d++) part->vel[d] += e[d] * factor;
        double x1[3], x2[3];
        for (int d = 0; d < 3; d++) {
            x1[d] = part->pos[d];
            x2[d] = part->pos[d] + part->vel[d] * dt;
            if (g->periodic[d]) {
                double L = g->xm[d] - g->x0[d];
                if (x2[d] < g->x0[d]) x2[d] += L;
                else if (x2[d] >= g->xm[d]) x2[d] -= L;
            }
        }
        int removed = !in_bounds(g, x2);
        if (!removed && in_object(g, x2)) {
            stats[0]++;
            obj_stream st = {{(uint32_t)ids[q], (uint32_t)(ids[q] >> 32), step, 0x0B000000u}, {seed_lo, seed_hi},
                             {0, 0, 0, 0}, 4};
            double t_rem = 1.0;
            int nb = 1;
            while (1) {
                int obj = in_object(g, x2);
                if (!obj) break;
                double tp, xi[3], nrm[3];
                box_line_intersect(g, obj - 1, x1, x2, &tp, xi, nrm);
                double vmag = len3(part->vel);
                if (charge == 0) {
                    reflect_vel(mass, vmag, nrm, draw_obj, &st, part->vel);
                    stats[1]++;
                    t_rem *= (1 - tp);
                    if (++nb > 20) {
                        removed = 1;
                        break;
                    }
                    for (int d = 0; d < 3; d++) {
                        x1[d] = xi[d];
                        x2[d] = xi[d] + part->vel[d] * t_rem * dt;
                        if (g->periodic[d]) {
                            double L = g->xm[d] - g->x0[d];
                            if (x2[d] < g->x0[d]) x2[d] += L;
                            else if (x2[d] >= g->xm[d]) x2[d] -= L;
                        }
                    }
                    if (!in_bounds(g, x2)) {
                        removed = 1;
                        break;
                    }
                    continue;
                }
                ion_impact(g, t, part->w, vmag, mass, xi, nrm, draw_obj, &st, 1, ids[q], step, stats + 2);
                removed = 1;
                break;
            }
        }
        if (removed) {
            p[q] = p[np - 1];
            ids[q] = ids[np - 1];
            np--;
            q--;
        } else {
            for (int d = 0; d < 3; d++) part->pos[d] = x2[d];
        }
    }
    return np;
}
