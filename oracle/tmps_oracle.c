/*
 * ORACLE — test infrastructure only.
 *
 * A plain-C, FP64 restatement of the reference (taichimps, Python + Taichi)
 * arithmetic for the per-step DEM contact path.  It exists to check the CUDA
 * product path: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it, and never as the thing measured or shipped.
 *
 * Built with -O2 -ffp-contract=off and no fast-math so every expression is
 * evaluated in the order the reference's Python/Taichi source writes it
 * (Taichi evaluates `a * b * c` as `(a * b) * c`, vector dot/norm as
 * `(e0 + e1) + e2`).  Each function names the reference file:line it follows.
 *
 * Layouts are the reference's: per-atom 3-vectors as [n][3] row-major
 * doubles, the half neighbor list as neighbors[n][max_nb] + num_neighbors[n],
 * the flat pair list pair_i/pair_j, and contact history per flat pair.
 *
 * Orthogonal boxes only: every configuration of the path has zero tilt; the
 * triclinic branches of domain.py are not restated.
 *
 * `nthreads > 1` runs the loops with OpenMP the way Taichi's CPU backend runs
 * its outermost loops (one iteration per thread, atomics on shared targets).
 * That variant is only used to time the CPU baseline; tests use nthreads = 1,
 * which makes the oracle deterministic.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    double lo[3];
    double hi[3];
    double prd[3];
    double h_rate[6];  /* [xprd, yprd, zprd, yz, xz, xy] rates (domain.py:64-67) */
    int32_t per[3];
    int32_t vremap;
} or_box_t;

typedef struct {
    /* legacy gran styles (hooke.py:29-50, hooke_history.py:86-106) */
    double kn, kt, gamman, gammat, xmu;
    int32_t limit_damping;
    /* pair granular (granular.py:122-205): model ids and derived coefficients */
    int32_t normal_id, damping_id, tangential_id;
    double damp, xt, mu;
    /* rolling resistance (GRANULAR/rolling.py:16-50): 0 none, 1 epsd */
    int32_t rolling_id;
    double k_roll, gamma_roll, mu_roll;
} or_pair_t;

enum { OR_HOOKE = 0, OR_HOOKE_HISTORY = 1, OR_HERTZ = 2, OR_HERTZ_HISTORY = 3, OR_GRANULAR = 4 };
/* granular.py:50-64 */
enum { N_HOOKE = 0, N_HERTZ = 1, N_HERTZ_MATERIAL = 2 };
enum { D_NONE = 0, D_VELOCITY = 1, D_MASS_VELOCITY = 2, D_VISCOELASTIC = 3, D_TSUJI = 4, D_COEFF_REST = 5 };
enum { T_NONE = 0, T_LINEAR_NOHISTORY = 1, T_LINEAR_HISTORY = 2, T_MINDLIN = 3 };

static int g_nthreads = 1;
void or_set_threads(int n) {
    g_nthreads = n < 1 ? 1 : n;
#ifdef _OPENMP
    omp_set_num_threads(g_nthreads);
#endif
}
int or_has_openmp(void) {
#ifdef _OPENMP
    return 1;
#else
    return 0;
#endif
}

/* ---------------------------------------------------------------- domain */

/* ti.round: round half away from zero (C round()).  Only exact half-box
 * separations depend on the tie rule; no reference test pins one. */
static inline double ti_round(double v) { return round(v); }

/* Domain.minimum_image_and_vshift, orthogonal branch (domain.py:388-447):
 * n = round(dx/prd) per periodic dim, dx -= n*prd, dv = n . h_rate when
 * remap v is on.  Returns dpos in d, the partner velocity shift in dv. */
static inline void min_image_vshift(const or_box_t* b, double d[3], double dv[3]) {
    double n[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < 3; ++k)
        if (b->per[k] == 1) n[k] = ti_round(d[k] / b->prd[k]);
    dv[0] = dv[1] = dv[2] = 0.0;
    if (b->vremap != 0) {
        const double* h = b->h_rate;
        dv[0] = (n[0] * h[0] + n[1] * h[5]) + n[2] * h[4];
        dv[1] = n[1] * h[1] + n[2] * h[3];
        dv[2] = n[2] * h[2];
    }
    /* apply_image_offsets, orthogonal (domain.py:455-457) */
    for (int k = 0; k < 3; ++k) d[k] -= n[k] * b->prd[k];
}

/* Domain.minimum_image, orthogonal branch (domain.py:481-486). */
static inline void min_image(const or_box_t* b, double d[3]) {
    for (int k = 0; k < 3; ++k)
        if (b->per[k] == 1) d[k] -= b->prd[k] * ti_round(d[k] / b->prd[k]);
}

/* Domain.pbc (domain.py:560-584): wrap, and under remap v add the velocity
 * kick of the crossing first (image_count domain.py:502-511, vremap_delta
 * domain.py:537-553, pbc_wrap domain.py:513-528). */
void or_pbc(const or_box_t* b, int n, double* x, double* v) {
#pragma omp parallel for if (g_nthreads > 1)
    for (int i = 0; i < n; ++i) {
        double* xi = x + 3 * i;
        if (b->vremap) {
            double c[3] = {0.0, 0.0, 0.0};
            for (int k = 0; k < 3; ++k) {
                double lam = (xi[k] - b->lo[k]) / b->prd[k];
                if (b->per[k] == 1) c[k] = floor(lam);
            }
            if (c[0] != 0.0 || c[1] != 0.0 || c[2] != 0.0) {
                const double* h = b->h_rate;
                double d0 = -((c[0] * h[0] + c[1] * h[5]) + c[2] * h[4]);
                double d1 = -(c[1] * h[1] + c[2] * h[3]);
                double d2 = -(c[2] * h[2]);
                v[3 * i + 0] += d0;
                v[3 * i + 1] += d1;
                v[3 * i + 2] += d2;
            }
        }
        for (int k = 0; k < 3; ++k) {
            if (b->per[k] == 1) {
                double s = (xi[k] - b->lo[k]) / b->prd[k];
                xi[k] = b->lo[k] + (s - floor(s)) * b->prd[k];
            }
        }
    }
}

/* ---------------------------------------------------------- neighbor list */

/* NeighborList.setup_grid (neighbor.py:143-189) with the orthogonal
 * perpendicular widths of neighbor.py:122-141 (vol / |b x c| etc.).
 * Returns the cell count. */
int or_setup_grid(const or_box_t* b, double max_cutoff, double skin, int max_cells,
                  int32_t gdim[3], double csize[3]) {
    double cut = max_cutoff + skin;
    if (cut <= 0) cut = 1.0;
    double xp = b->prd[0], yp = b->prd[1], zp = b->prd[2];
    double vol = xp * yp * zp;
    double w[3];
    w[0] = vol / fabs(yp * zp);
    w[1] = vol / fabs(zp * xp);
    w[2] = vol / fabs(xp * yp);
    long g[3];
    for (int k = 0; k < 3; ++k) {
        double q = floor(w[k] / cut);
        g[k] = (long)q;
        if (g[k] < 1) g[k] = 1;
        if (b->per[k] == 1 && g[k] == 2) g[k] = 1;
    }
    double total = (double)g[0] * (double)g[1] * (double)g[2];
    if (total > (double)max_cells) {
        double factor = pow((double)max_cells / total, 1.0 / 3.0);
        for (int k = 0; k < 3; ++k) {
            long s = (long)((double)g[k] * factor);
            g[k] = s < 1 ? 1 : s;
        }
    }
    for (int k = 0; k < 3; ++k) {
        gdim[k] = (int32_t)g[k];
        csize[k] = 1.0 / (double)g[k];
    }
    return (int)(g[0] * g[1] * g[2]);
}

/* NeighborList.get_cell_coord (neighbor.py:191-206): bin in lamda
 * coordinates, floor(lamda / csize), clamped to the grid. */
static inline void cell_coord(const or_box_t* b, const int32_t g[3], const double cs[3],
                              const double* x, int32_t c[3]) {
    for (int k = 0; k < 3; ++k) {
        double lam = (x[k] - b->lo[k]) / b->prd[k];
        int32_t ck = (int32_t)floor(lam / cs[k]);
        if (ck > g[k] - 1) ck = g[k] - 1;
        if (ck < 0) ck = 0;
        c[k] = ck;
    }
}

/* NeighborList.build_grid (neighbor.py:247-282): counting sort.  Members
 * of a cell are placed in atom-index order (the reference's order is
 * whatever its atomics hand out, which only permutes a neighbor row). */
void or_build_grid(const or_box_t* b, const int32_t g[3], const double cs[3], int n,
                   const double* x, int32_t* cell_of, int32_t* cell_start,
                   int32_t* cell_particles) {
    int gx = g[0], gxy = g[0] * g[1];
    int ncell = gxy * g[2];
    for (int c = 0; c <= ncell; ++c) cell_start[c] = 0;
    for (int i = 0; i < n; ++i) {
        int32_t c3[3];
        cell_coord(b, g, cs, x + 3 * i, c3);
        int ci = c3[0] + c3[1] * gx + c3[2] * gxy;
        cell_of[i] = ci;
        cell_start[ci + 1] += 1;
    }
    for (int c = 0; c < ncell; ++c) cell_start[c + 1] += cell_start[c];
    int32_t* fill = (int32_t*)calloc((size_t)(ncell > 0 ? ncell : 0) + 1, sizeof(int32_t));
    for (int i = 0; i < n; ++i) {
        int c = cell_of[i];
        cell_particles[cell_start[c] + fill[c]++] = i;
    }
    free(fill);
}

/* NeighborList.build_neighbor_list (neighbor.py:305-369): 27-cell stencil
 * (dx outermost, dz innermost), periodic wrap with the single-bin skip
 * rule, half list j > i, cut (ri + rj + skin)^2.  Returns 1 on overflow. */
int or_build_neighbor_list(const or_box_t* b, const int32_t g[3], const double cs[3], int n,
                           const double* x, const double* radius, double skin,
                           const int32_t* cell_start, const int32_t* cell_particles,
                           int max_nb, int32_t* num_neighbors, int32_t* neighbors) {
    int gx = g[0], gy = g[1], gz = g[2], gxy = gx * gy;
    int overflow = 0;
#pragma omp parallel for if (g_nthreads > 1) reduction(| : overflow)
    for (int i = 0; i < n; ++i) {
        const double* xi = x + 3 * i;
        double ri = radius[i];
        int32_t c3[3];
        cell_coord(b, g, cs, xi, c3);
        int count = 0;
        for (int ox = -1; ox <= 1; ++ox)
            for (int oy = -1; oy <= 1; ++oy)
                for (int oz = -1; oz <= 1; ++oz) {
                    int nx = c3[0] + ox, ny = c3[1] + oy, nz = c3[2] + oz;
                    int skip = (b->per[0] == 1 && gx == 1 && ox != 0) ||
                               (b->per[1] == 1 && gy == 1 && oy != 0) ||
                               (b->per[2] == 1 && gz == 1 && oz != 0);
                    if (b->per[0] == 1) nx = (nx % gx + gx) % gx;
                    if (b->per[1] == 1) ny = (ny % gy + gy) % gy;
                    if (b->per[2] == 1) nz = (nz % gz + gz) % gz;
                    if (skip || nx < 0 || nx >= gx || ny < 0 || ny >= gy || nz < 0 || nz >= gz)
                        continue;
                    int c = nx + ny * gx + nz * gxy;
                    for (int p = cell_start[c]; p < cell_start[c + 1]; ++p) {
                        int j = cell_particles[p];
                        if (j <= i) continue;
                        double d[3] = {xi[0] - x[3 * j], xi[1] - x[3 * j + 1], xi[2] - x[3 * j + 2]};
                        min_image(b, d);
                        double rsq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
                        double rad = (ri + radius[j]) + skin;
                        if (rsq < rad * rad) {
                            if (count < max_nb) {
                                neighbors[(size_t)i * max_nb + count] = j;
                                count += 1;
                            } else {
                                overflow = 1;
                            }
                        }
                    }
                }
        num_neighbors[i] = count;
    }
    return overflow;
}

/* NeighborList.build_pair_list (neighbor.py:284-303).  Returns npairs. */
int or_build_pair_list(int n, int max_nb, const int32_t* num_neighbors, const int32_t* neighbors,
                       int32_t* pair_start, int32_t* pair_i, int32_t* pair_j) {
    pair_start[0] = 0;
    for (int i = 0; i < n; ++i) pair_start[i + 1] = pair_start[i] + num_neighbors[i];
    for (int i = 0; i < n; ++i) {
        int base = pair_start[i];
        for (int k = 0; k < num_neighbors[i]; ++k) {
            pair_i[base + k] = i;
            pair_j[base + k] = neighbors[(size_t)i * max_nb + k];
        }
    }
    return pair_start[n];
}

/* NeighborList.check_displacement (neighbor.py:214-245): 1 when any atom
 * moved more than half the skin since x0 was stored. */
/* ComputeContactAtom.compute_kernel (computes/contact_atom.py:21-52): over the
 * half list, every pair with rsq < (ri + rj)^2 and rsq > 1e-18 counts for both
 * of its atoms. */
void or_contact_count(const or_box_t* b, int n, const double* x, const double* radius, int max_nb,
                      const int32_t* num_neighbors, const int32_t* neighbors, int32_t* count) {
    for (int i = 0; i < n; ++i) count[i] = 0;
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < num_neighbors[i]; ++k) {
            const int j = neighbors[(size_t)i * max_nb + k];
            double d[3] = {x[3 * i] - x[3 * j], x[3 * i + 1] - x[3 * j + 1], x[3 * i + 2] - x[3 * j + 2]};
            min_image(b, d);
            const double rsq = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2];
            const double radsum = radius[i] + radius[j];
            if (rsq < radsum * radsum && rsq > 1e-18) {
                count[i] += 1;
                count[j] += 1;
            }
        }
    }
}

int or_skin_check(int n, const double* x, const double* x0, double trigger_sq) {
    int hit = 0;
#pragma omp parallel for if (g_nthreads > 1) reduction(| : hit)
    for (int i = 0; i < n; ++i) {
        double d0 = x[3 * i] - x0[3 * i], d1 = x[3 * i + 1] - x0[3 * i + 1],
               d2 = x[3 * i + 2] - x0[3 * i + 2];
        if ((d0 * d0 + d1 * d1) + d2 * d2 > trigger_sq) hit = 1;
    }
    return hit;
}

/* ---------------------------------------------------------- contact history */

/* ContactHistory.save_state_kernel (contact_history.py:91-110): compact the
 * touching pairs (partner >= 0) into tag-keyed per-atom buffers. */
void or_history_save(int n, int npairs, const int32_t* pair_i, const int32_t* partner,
                     const double* shear, const double* rolling, int max_nb, int32_t* save_count,
                     int32_t* save_tag, double* save_shear, double* save_rolling) {
    for (int i = 0; i < n; ++i) save_count[i] = 0;
    for (int nc = 0; nc < npairs; ++nc) {
        int32_t ptag = partner[nc];
        if (ptag >= 0) {
            int i = pair_i[nc];
            int m = save_count[i]++;
            save_tag[(size_t)i * max_nb + m] = ptag;
            for (int k = 0; k < 3; ++k) save_shear[((size_t)i * max_nb + m) * 3 + k] = shear[3 * nc + k];
            if (rolling)
                for (int k = 0; k < 3; ++k) save_rolling[((size_t)i * max_nb + m) * 3 + k] = rolling[3 * nc + k];
        }
    }
}

/* ContactHistory.restore_state_kernel (contact_history.py:112-139): look the
 * partner's tag up in the saved buffer of atom i; copy or zero. */
void or_history_restore(int npairs, const int32_t* pair_i, const int32_t* pair_j, const int32_t* tag,
                        int max_nb, const int32_t* save_count, const int32_t* save_tag,
                        const double* save_shear, const double* save_rolling, int32_t* partner,
                        double* shear, double* rolling) {
    for (int nc = 0; nc < npairs; ++nc) {
        int i = pair_i[nc];
        int32_t jtag = tag[pair_j[nc]];
        int found = -1;
        for (int m = 0; m < save_count[i]; ++m)
            if (save_tag[(size_t)i * max_nb + m] == jtag) { found = m; break; }
        if (found >= 0) {
            partner[nc] = jtag;
            for (int k = 0; k < 3; ++k) shear[3 * nc + k] = save_shear[((size_t)i * max_nb + found) * 3 + k];
            if (rolling)
                for (int k = 0; k < 3; ++k) rolling[3 * nc + k] = save_rolling[((size_t)i * max_nb + found) * 3 + k];
        } else {
            partner[nc] = -1;
            shear[3 * nc] = shear[3 * nc + 1] = shear[3 * nc + 2] = 0.0;
            if (rolling) rolling[3 * nc] = rolling[3 * nc + 1] = rolling[3 * nc + 2] = 0.0;
        }
    }
}

/* ---------------------------------------------------------- pair styles */

static inline double dot3(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static inline double norm3(const double* a) { return sqrt(dot3(a, a)); }
/* Taichi Vector.cross: [a1 b2 - a2 b1, a2 b0 - a0 b2, a0 b1 - a1 b0] */
static inline void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static inline void add3(double* dst, const double* v, double s) {
    /* dst += s * v, one component at a time; atomics when threaded */
    for (int k = 0; k < 3; ++k) {
        double t = s * v[k];
#pragma omp atomic
        dst[k] += t;
    }
}
static inline void add_raw(double* dst, const double* v, int m) {
    for (int k = 0; k < m; ++k) {
#pragma omp atomic
        dst[k] += v[k];
    }
}

/* GranSubMod::rotate_rescale_vec as granular.py:271-280 restates it. */
static inline void rotate_rescale(double* vec, const double* n) {
    double shrmag = norm3(vec);
    double rsht = dot3(vec, n);
    double out[3];
    for (int k = 0; k < 3; ++k) out[k] = vec[k] - rsht * n[k];
    double prjmag = norm3(out);
    double scale = 0.0;
    if (prjmag > 0.0) scale = shrmag / prjmag;
    for (int k = 0; k < 3; ++k) vec[k] = out[k] * scale;
}

/*
 * One contact of every pair style, in the i -> j orientation of the half
 * list.  Follows, operation for operation:
 *   OR_HOOKE          hooke.py:65-155
 *   OR_HOOKE_HISTORY  hooke_history.py:71-195
 *   OR_HERTZ          hertz.py:59-130
 *   OR_HERTZ_HISTORY  hertz_history.py:74-171
 *   OR_GRANULAR       granular.py:303-430
 */
static void pair_one(int style, const or_pair_t* P, const or_box_t* b, int nc, int i, int j,
                     const double* x, const double* v, const double* om, const double* rad,
                     const double* rmass, const int32_t* tag, int32_t* partner, double* shear,
                     double* rolling, double dt, int shearupdate, double* f, double* torque,
                     double* virial) {
    const double* xi = x + 3 * i; const double* xj = x + 3 * j;
    const double* vi = v + 3 * i; const double* vj = v + 3 * j;
    const double* oi = om + 3 * i; const double* oj = om + 3 * j;
    double ri = rad[i], rj = rad[j], mi = rmass[i], mj = rmass[j];
    int has_rolling = style == OR_GRANULAR && P->rolling_id != 0 && rolling != NULL;
    int has_hist = style == OR_HOOKE_HISTORY || style == OR_HERTZ_HISTORY ||
                   (style == OR_GRANULAR &&
                    (P->tangential_id == T_LINEAR_HISTORY || P->tangential_id == T_MINDLIN)) ||
                   has_rolling;

    double dpos[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
    double dvj[3];
    min_image_vshift(b, dpos, dvj);
    double rsq = dot3(dpos, dpos);
    double radsum = ri + rj;
    if (!(rsq < radsum * radsum && rsq > 1e-28)) {
        if (has_hist) {
            partner[nc] = -1;
            shear[3 * nc] = shear[3 * nc + 1] = shear[3 * nc + 2] = 0.0;
            if (has_rolling) rolling[3 * nc] = rolling[3 * nc + 1] = rolling[3 * nc + 2] = 0.0;
        }
        return;
    }
    double ftot[3], fs[3], tor[3], troll[3] = {0.0, 0.0, 0.0};
    double armi, armj;  /* torque prefactors applied to tor */

    if (style != OR_GRANULAR) {
        double r = sqrt(rsq);
        double delta = radsum - r;
        double polyhertz = 1.0;
        int hertz = style == OR_HERTZ || style == OR_HERTZ_HISTORY;
        if (hertz) {
            double reff = (ri * rj) / (ri + rj);
            polyhertz = sqrt(reff * delta);
        }
        double meff = (mi * mj) / (mi + mj);
        double rsqinv = 1.0 / rsq;
        double rinv = 1.0 / r;
        double vrel_t[3], vn[3], vt[3], wr[3], cr[3], vtr[3];
        for (int k = 0; k < 3; ++k) vrel_t[k] = vi[k] - (vj[k] + dvj[k]);
        double vnnr = dot3(vrel_t, dpos);
        double s = vnnr * rsqinv;
        for (int k = 0; k < 3; ++k) vn[k] = dpos[k] * s;
        for (int k = 0; k < 3; ++k) vt[k] = vrel_t[k] - vn[k];
        for (int k = 0; k < 3; ++k) wr[k] = (ri * oi[k] + rj * oj[k]) * rinv;
        cross3(dpos, wr, cr);
        for (int k = 0; k < 3; ++k) vtr[k] = vt[k] + cr[k];
        double damp = ((meff * P->gamman) * vnnr) * rsqinv;
        double ccel = (P->kn * delta) * rinv - damp;
        if (hertz) ccel = ccel * polyhertz;
        if (P->limit_damping == 1 && ccel < 0.0) ccel = 0.0;

        if (style == OR_HOOKE || style == OR_HERTZ) {
            double vrel = norm3(vtr);
            double fn = P->xmu * fabs(ccel * r);
            double fsd = (meff * P->gammat) * vrel;
            double ft = 0.0;
            if (vrel > 1e-16) ft = (fn < fsd ? fn : fsd) / vrel;
            for (int k = 0; k < 3; ++k) fs[k] = (-ft) * vtr[k];
        } else {
            int32_t jtag = tag[j];
            double sh[3] = {shear[3 * nc], shear[3 * nc + 1], shear[3 * nc + 2]};
            if (partner[nc] != jtag) {
                sh[0] = sh[1] = sh[2] = 0.0;
                partner[nc] = jtag;
            }
            double geff = meff * P->gammat;
            if (shearupdate != 0)
                for (int k = 0; k < 3; ++k) sh[k] = sh[k] + vtr[k] * dt;
            double shrmag = norm3(sh);
            if (shearupdate != 0) {
                double rsht = dot3(sh, dpos) * rsqinv;
                for (int k = 0; k < 3; ++k) sh[k] = sh[k] - rsht * dpos[k];
            }
            for (int k = 0; k < 3; ++k) {
                double t = P->kt * sh[k] + geff * vtr[k];
                fs[k] = hertz ? (-polyhertz) * t : -t;
            }
            double fsmag = norm3(fs);
            double fn = P->xmu * fabs(ccel * r);
            if (fsmag > fn) {
                if (shrmag != 0.0) {
                    double ratio = fn / fsmag;
                    for (int k = 0; k < 3; ++k) {
                        double dc = (geff * vtr[k]) / P->kt;
                        sh[k] = ratio * (sh[k] + dc) - dc;
                        fs[k] = ratio * fs[k];
                    }
                } else {
                    fs[0] = fs[1] = fs[2] = 0.0;
                }
            }
            shear[3 * nc] = sh[0]; shear[3 * nc + 1] = sh[1]; shear[3 * nc + 2] = sh[2];
        }
        for (int k = 0; k < 3; ++k) ftot[k] = dpos[k] * ccel + fs[k];
        double c[3];
        cross3(dpos, fs, c);
        for (int k = 0; k < 3; ++k) tor[k] = rinv * c[k];
        armi = -ri; armj = -rj;
    } else {
        double r = sqrt(rsq);
        double rinv = 1.0 / r;
        double n[3] = {dpos[0] * rinv, dpos[1] * rinv, dpos[2] * rinv};
        double delta = radsum - r;
        double reff = (ri * rj) / radsum;
        double meff = (mi * mj) / (mi + mj);
        double a = sqrt(delta * reff);
        double vr[3], vt[3], wr[3], cr[3], vtr[3];
        for (int k = 0; k < 3; ++k) vr[k] = vi[k] - (vj[k] + dvj[k]);
        double vnnr = dot3(vr, n);
        for (int k = 0; k < 3; ++k) vt[k] = vr[k] - vnnr * n[k];
        for (int k = 0; k < 3; ++k) wr[k] = ri * oi[k] + rj * oj[k];
        cross3(wr, n, cr);
        for (int k = 0; k < 3; ++k) vtr[k] = vt[k] - cr[k];
        double vrel = norm3(vtr);
        double fne = (P->normal_id != N_HOOKE) ? (P->kn * a) * delta : P->kn * delta;
        double dpf = 0.0;
        switch (P->damping_id) {
            case D_VELOCITY: dpf = P->damp; break;
            case D_MASS_VELOCITY: dpf = P->damp * meff; break;
            case D_VISCOELASTIC: dpf = (P->damp * meff) * a; break;
            case D_TSUJI:
            case D_COEFF_REST: {
                double arg = 0.0;
                if (delta > 0.0) {
                    double q = (meff * fne) / delta;
                    arg = q > 0.0 ? q : 0.0;
                }
                dpf = P->damp * sqrt(arg);
                break;
            }
            default: dpf = 0.0;
        }
        double fntot = fne - dpf * vnnr;
        if (P->limit_damping == 1 && fntot < 0.0) fntot = 0.0;
        double fscrit = P->mu * fabs(fntot);
        fs[0] = fs[1] = fs[2] = 0.0;
        /* a slot whose partner changed starts from zero history (shear and rolling) */
        const int fresh = has_hist && partner[nc] != tag[j];
        if (P->tangential_id == T_LINEAR_NOHISTORY) {
            double damp_t = P->xt * dpf;
            double ft = 0.0;
            if (vrel != 0.0) {
                double q = damp_t * vrel;
                ft = (fscrit < q ? fscrit : q) / vrel;
            }
            for (int k = 0; k < 3; ++k) fs[k] = (-ft) * vtr[k];
        } else if (P->tangential_id == T_LINEAR_HISTORY || P->tangential_id == T_MINDLIN) {
            int32_t jtag = tag[j];
            double h[3] = {shear[3 * nc], shear[3 * nc + 1], shear[3 * nc + 2]};
            if (fresh) {
                h[0] = h[1] = h[2] = 0.0;
                partner[nc] = jtag;
            }
            double keff = P->kt;
            if (P->tangential_id == T_MINDLIN) keff = P->kt * a;
            double damp_t = P->xt * dpf;
            if (shearupdate != 0) {
                double rsht = dot3(h, n);
                if (fabs(rsht) * keff > 1e-10 * fscrit) rotate_rescale(h, n);
                for (int k = 0; k < 3; ++k) h[k] = h[k] + vtr[k] * dt;
            }
            double fdamp[3];
            for (int k = 0; k < 3; ++k) fdamp[k] = (-damp_t) * vtr[k];
            for (int k = 0; k < 3; ++k) fs[k] = (-keff) * h[k] + fdamp[k];
            double magfs = norm3(fs);
            if (magfs > fscrit) {
                if (norm3(h) != 0.0) {
                    double sc = fscrit / magfs;
                    for (int k = 0; k < 3; ++k) fs[k] = fs[k] * sc;
                    for (int k = 0; k < 3; ++k) h[k] = (-(fs[k] - fdamp[k])) / keff;
                } else {
                    fs[0] = fs[1] = fs[2] = 0.0;
                }
            }
            shear[3 * nc] = h[0]; shear[3 * nc + 1] = h[1]; shear[3 * nc + 2] = h[2];
        }
        if (has_rolling) {
            /* RollingResistance.compute_torque (rolling.py:30-50) with omega_rel = omega_i - omega_j,
             * r_eff the effective radius and fn = |fntot|; the increment only on a history update */
            double hr[3] = {rolling[3 * nc], rolling[3 * nc + 1], rolling[3 * nc + 2]};
            if (fresh) {
                hr[0] = hr[1] = hr[2] = 0.0;
                partner[nc] = tag[j];
            }
            double wrel[3] = {oi[0] - oj[0], oi[1] - oj[1], oi[2] - oj[2]};
            if (shearupdate != 0)
                for (int k = 0; k < 3; ++k) hr[k] = hr[k] + wrel[k] * dt;
            const double tr_mag = P->k_roll * norm3(hr);
            const double tr_max = (P->mu_roll * reff) * fabs(fntot);
            for (int k = 0; k < 3; ++k) troll[k] = (-P->k_roll) * hr[k] - P->gamma_roll * wrel[k];
            if (tr_mag > tr_max && tr_mag > 1e-12) {
                for (int k = 0; k < 3; ++k) {
                    troll[k] = (-tr_max) * (hr[k] / tr_mag);
                    hr[k] = (tr_max / P->k_roll) * (hr[k] / tr_mag);
                }
            }
            rolling[3 * nc] = hr[0]; rolling[3 * nc + 1] = hr[1]; rolling[3 * nc + 2] = hr[2];
        }
        for (int k = 0; k < 3; ++k) ftot[k] = fntot * n[k] + fs[k];
        double c[3];
        cross3(n, fs, c);
        for (int k = 0; k < 3; ++k) tor[k] = -c[k];
        armi = ri - 0.5 * delta;
        armj = rj - 0.5 * delta;
    }

    add3(f + 3 * i, ftot, 1.0);
    add3(f + 3 * j, ftot, -1.0);
    add3(torque + 3 * i, tor, armi);
    add3(torque + 3 * j, tor, armj);
    add3(torque + 3 * i, troll, 1.0);
    add3(torque + 3 * j, troll, -1.0);
    /* Pair::ev_tally_xyz as restated at hooke_history.py:181-191 */
    double vir[6] = {0.5 * (dpos[0] * ftot[0]), 0.5 * (dpos[1] * ftot[1]), 0.5 * (dpos[2] * ftot[2]),
                     0.5 * (dpos[0] * ftot[1]), 0.5 * (dpos[0] * ftot[2]), 0.5 * (dpos[1] * ftot[2])};
    add_raw(virial + 6 * i, vir, 6);
    add_raw(virial + 6 * j, vir, 6);
}

/* GranularPair.compute for every style: one iteration per flat pair. */
void or_pair_compute(int style, const or_pair_t* P, const or_box_t* b, int npairs,
                     const int32_t* pair_i, const int32_t* pair_j, const double* x, const double* v,
                     const double* om, const double* rad, const double* rmass, const int32_t* tag,
                     int32_t* partner, double* shear, double* rolling, double dt, int shearupdate,
                     double* f, double* torque, double* virial) {
#pragma omp parallel for if (g_nthreads > 1) schedule(static)
    for (int nc = 0; nc < npairs; ++nc)
        pair_one(style, P, b, nc, pair_i[nc], pair_j[nc], x, v, om, rad, rmass, tag, partner, shear,
                 rolling, dt, shearupdate, f, torque, virial);
}

/* ---------------------------------------------------------- fixes */

/* AtomSystem._clear_forces_kernel (atom.py:201-206) */
void or_clear_forces(int n, double* f, double* torque, double* virial) {
    memset(f, 0, sizeof(double) * 3 * (size_t)n);
    memset(torque, 0, sizeof(double) * 3 * (size_t)n);
    memset(virial, 0, sizeof(double) * 6 * (size_t)n);
}

/* FixNVESphere.initial_integrate_kernel (nve_sphere.py:44-77) */
void or_nve_initial(int n, double dt, double* x, double* v, double* om, const double* f,
                    const double* torque, const double* rad, const double* rmass) {
#pragma omp parallel for if (g_nthreads > 1)
    for (int i = 0; i < n; ++i) {
        double dtv = dt, dtf = 0.5 * dt;
        double m = rmass[i], r = rad[i];
        double inertia = ((0.4 * m) * r) * r;
        for (int k = 0; k < 3; ++k) v[3 * i + k] += dtf * (f[3 * i + k] / m);
        for (int k = 0; k < 3; ++k) x[3 * i + k] = x[3 * i + k] + dtv * v[3 * i + k];
        for (int k = 0; k < 3; ++k) om[3 * i + k] += dtf * (torque[3 * i + k] / inertia);
    }
}

/* FixNVESphere.final_integrate_kernel (nve_sphere.py:79-96) */
void or_nve_final(int n, double dt, double* v, double* om, const double* f, const double* torque,
                  const double* rad, const double* rmass) {
#pragma omp parallel for if (g_nthreads > 1)
    for (int i = 0; i < n; ++i) {
        double dtf = 0.5 * dt;
        double m = rmass[i], r = rad[i];
        double inertia = ((0.4 * m) * r) * r;
        for (int k = 0; k < 3; ++k) v[3 * i + k] += dtf * (f[3 * i + k] / m);
        for (int k = 0; k < 3; ++k) om[3 * i + k] += dtf * (torque[3 * i + k] / inertia);
    }
}

/* FixDampingCundall.post_force_kernel (damping_cundall.py:36-53) */
void or_cundall(int n, double gl, double ga, double* f, double* torque, const double* v, const double* om) {
#pragma omp parallel for if (g_nthreads > 1)
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            double wl = f[3 * i + d] * v[3 * i + d];
            double sf = wl >= 0.0 ? 1.0 : -1.0;
            f[3 * i + d] *= 1.0 - gl * sf;
            double wa = torque[3 * i + d] * om[3 * i + d];
            double st = wa >= 0.0 ? 1.0 : -1.0;
            torque[3 * i + d] *= 1.0 - ga * st;
        }
}

/* Computes.compute_virial_kernel (thermo.py:62-109): chunked strided
 * partial sums, then a serial sum over chunks per component. */
void or_virial(int n, const double* virial, const double* v, const double* rmass, int keflag,
               int chunks, double out[6]) {
    double* part = (double*)calloc((size_t)chunks * 6, sizeof(double));
#pragma omp parallel for if (g_nthreads > 1)
    for (int c = 0; c < chunks; ++c) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int i = c; i < n; i += chunks) {
            for (int k = 0; k < 6; ++k) acc[k] += virial[6 * i + k];
            if (keflag != 0) {
                double m = rmass[i];
                const double* vi = v + 3 * i;
                acc[0] += (m * vi[0]) * vi[0];
                acc[1] += (m * vi[1]) * vi[1];
                acc[2] += (m * vi[2]) * vi[2];
                acc[3] += (m * vi[0]) * vi[1];
                acc[4] += (m * vi[0]) * vi[2];
                acc[5] += (m * vi[1]) * vi[2];
            }
        }
        for (int k = 0; k < 6; ++k) part[6 * c + k] = acc[k];
    }
    for (int k = 0; k < 6; ++k) {
        double t = 0.0;
        for (int c = 0; c < chunks; ++c) t += part[6 * c + k];
        out[k] = t;
    }
    free(part);
}

/* FixDeformPressure.remap_positions, orthogonal (deform_pressure.py:493-530):
 * lamda with the old box, back with the new one, anchored on the new lo. */
void or_remap_x(int n, double* x, const double old_lo[3], const double old_prd[3],
                const double new_lo[3], const double new_prd[3]) {
#pragma omp parallel for if (g_nthreads > 1)
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            double d = x[3 * i + k] - old_lo[k];
            double lam = d / old_prd[k];
            x[3 * i + k] = new_prd[k] * lam + new_lo[k];
        }
}

/* Granular walls.  FixWallGran.post_force_kernel (EXTRA_FIX/wall_gran.py:143-228)
 * for kind 0 (plane) and FixWallGranRegion.post_force_kernel
 * (EXTRA_FIX/wall_gran_region.py:134-276) for kind 1 (cylinder side); every
 * expression in the reference's order.  Per-atom history shear[n][3],
 * touch[n]. */
typedef struct or_wall_t {
    int kind, axis, side, history, hertz, limit_damping, shear_axis, has_axis_bounds;
    double coord, vwall_n, vwall_s, c1, c2, radius, axis_lo, axis_hi;
    double kn, kt, gamman, gammat, xmu;
} or_wall_t;

static double wdot(const double* a, const double* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static void wcross(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* linear_history_classic (with the cylinder's contact-radius factor) or the
 * history-free dashpot with the Coulomb cap */
static void wall_tangential(const or_wall_t* P, double dt, int upd, const double* n, const double* vtr, double vrel,
                            double fscrit, double damp_t, double poly, double* sh, int* touch, double* fs) {
    if (P->history) {
        double hist[3] = {sh[0], sh[1], sh[2]}, fdamp[3];
        if (*touch == 0) {
            hist[0] = hist[1] = hist[2] = 0.0;
            *touch = 1;
        }
        if (upd)
            for (int k = 0; k < 3; ++k) hist[k] = hist[k] + vtr[k] * dt;
        double shrmag = sqrt(wdot(hist, hist));
        if (upd) {
            double hn = wdot(hist, n);
            for (int k = 0; k < 3; ++k) hist[k] = hist[k] - hn * n[k];
        }
        for (int k = 0; k < 3; ++k) {
            fdamp[k] = -damp_t * vtr[k];
            fs[k] = P->kind == 0 ? -P->kt * hist[k] + fdamp[k] : (-P->kt * poly) * hist[k] + fdamp[k];
        }
        double magfs = sqrt(wdot(fs, fs));
        if (magfs > fscrit) {
            if (shrmag != 0.0) {
                double s = fscrit / magfs, kk = P->kind == 0 ? P->kt : P->kt * poly;
                for (int k = 0; k < 3; ++k) {
                    fs[k] = fs[k] * s;
                    hist[k] = -(fs[k] - fdamp[k]) / kk;
                }
            } else {
                fs[0] = fs[1] = fs[2] = 0.0;
            }
        }
        for (int k = 0; k < 3; ++k) sh[k] = hist[k];
    } else {
        double ft = 0.0;
        if (vrel != 0.0) ft = fmin(fscrit, damp_t * vrel) / vrel;
        for (int k = 0; k < 3; ++k) fs[k] = -ft * vtr[k];
    }
}

void or_wall(const or_wall_t* P, int n, double dt, int upd, const double* x, const double* v, const double* om,
             const double* radius, const double* rmass, double* f, double* torque, double* shear, int32_t* touch_) {
    for (int i = 0; i < n; ++i) {
        const double* xi = x + 3 * i;
        const double* vi = v + 3 * i;
        const double* wi = om + 3 * i;
        double ri = radius[i], mi = rmass[i];
        double sh[3] = {0, 0, 0};
        int touch = 0;
        if (P->history) {
            for (int k = 0; k < 3; ++k) sh[k] = shear[3 * i + k];
            touch = touch_[i];
        }
        int contact = 0;
        double F[3] = {0, 0, 0}, T[3] = {0, 0, 0};
        if (P->kind == 0) {
            double nrm[3] = {0, 0, 0}, vwall[3] = {0, 0, 0};
            nrm[P->axis] = P->side == 1 ? -1.0 : 1.0;
            vwall[P->axis] = P->vwall_n;
            if (P->shear_axis >= 0) vwall[P->shear_axis] = P->vwall_s;
            double dist = P->side == -1 ? xi[P->axis] - P->coord : P->coord - xi[P->axis];
            double delta = ri - dist;
            if (delta > 0.0) {
                contact = 1;
                double vr[3], vt[3], wr[3], c[3], vtr[3], fs[3], nf[3];
                for (int k = 0; k < 3; ++k) vr[k] = vi[k] - vwall[k];
                double vnnr = wdot(vr, nrm);
                for (int k = 0; k < 3; ++k) {
                    vt[k] = vr[k] - vnnr * nrm[k];
                    wr[k] = ri * wi[k];
                }
                wcross(wr, nrm, c);
                for (int k = 0; k < 3; ++k) vtr[k] = vt[k] - c[k];
                double vrel = sqrt(wdot(vtr, vtr));
                double damp_prefactor = mi * P->gamman;
                double fntot = P->kn * delta - damp_prefactor * vnnr;
                if (P->limit_damping == 1) fntot = fmax(fntot, 0.0);
                double fscrit = P->xmu * fabs(fntot);
                double damp_t = mi * P->gammat;
                wall_tangential(P, dt, upd, nrm, vtr, vrel, fscrit, damp_t, 1.0, sh, &touch, fs);
                wcross(nrm, fs, nf);
                for (int k = 0; k < 3; ++k) {
                    F[k] = fntot * nrm[k] + fs[k];
                    T[k] = -ri * nf[k];
                }
            }
        } else {
            double pa = xi[P->axis];
            if (!(P->has_axis_bounds == 1 && (pa < P->axis_lo || pa > P->axis_hi))) {
                int a1 = P->axis == 0 ? 1 : 0, a2 = P->axis == 2 ? 1 : 2;
                double d1 = xi[a1] - P->c1, d2 = xi[a2] - P->c2;
                double r_perp = sqrt(d1 * d1 + d2 * d2);
                if (r_perp > 1e-14) {
                    double inv = 1.0 / r_perp, u1 = d1 * inv, u2 = d2 * inv;
                    double sg = P->side == -1 ? -1.0 : 1.0;
                    double nrm[3] = {0, 0, 0};
                    nrm[a1] = sg * u1;
                    nrm[a2] = sg * u2;
                    double delta = P->side == -1 ? ri - (P->radius - r_perp) : ri - (r_perp - P->radius);
                    if (delta > 0.0) {
                        contact = 1;
                        double c[3], vr[3], vrt[3], fs[3], nf[3];
                        wcross(wi, nrm, c);
                        for (int k = 0; k < 3; ++k) vr[k] = vi[k] - ri * c[k];
                        double vn = wdot(vr, nrm);
                        for (int k = 0; k < 3; ++k) vrt[k] = vr[k] - vn * nrm[k];
                        double vrel = sqrt(wdot(vrt, vrt));
                        double poly = P->hertz ? sqrt(ri * delta) : 1.0;
                        double fn_elastic = P->kn * delta * poly;
                        double damp_prefactor = mi * P->gamman * poly;
                        double fntot = fn_elastic - damp_prefactor * vn;
                        if (P->limit_damping == 1) fntot = fmax(fntot, 0.0);
                        double fscrit = P->xmu * fabs(fntot);
                        double damp_t = mi * P->gammat * poly;
                        wall_tangential(P, dt, upd, nrm, vrt, vrel, fscrit, damp_t, poly, sh, &touch, fs);
                        wcross(nrm, fs, nf);
                        for (int k = 0; k < 3; ++k) {
                            F[k] = fntot * nrm[k] + fs[k];
                            T[k] = -ri * nf[k];
                        }
                    }
                }
            }
        }
        if (contact) {
            for (int k = 0; k < 3; ++k) {
                f[3 * i + k] += F[k];
                torque[3 * i + k] += T[k];
            }
        } else {
            touch = 0;
            sh[0] = sh[1] = sh[2] = 0.0;
        }
        if (P->history) {
            for (int k = 0; k < 3; ++k) shear[3 * i + k] = sh[k];
            touch_[i] = touch;
        }
    }
}
