/*
 * csmc_oracle.c -- CPU FP64 oracle for the ClassicalSpinMC.jl hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see csmc_oracle.h): the parity checker for the
 * GPU library and the timed CPU baseline of bench.py.  Every routine cites
 * the reference routine it restates (paths within the ClassicalSpinMC.jl
 * project).  Build with -O2 -ffp-contract=off so that no a*b+c is fused:
 * Julia evaluates left to right without contraction.
 */
#include "csmc_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct orc_lattice {
    int D, nb, shape[3], periodic;
    double S;
    int64_t N, cells;
    int N2, N3, N4;
    int32_t *idx;      /* N x (1+D): (b, n1..nD), 1-based, sorted (lattice.jl:29-33) */
    double *field;     /* N x 3 */
    double *onsite;    /* N x 9 */
    int64_t *bsites;   /* N x N2, 0-based, -1 = absent */
    double *bmats;     /* N x N2 x 9 */
    int64_t *csites;   /* N x N3 x 2 */
    double *ctens;     /* N x N3 x 27 */
    int64_t *qsites;   /* N x N4 x 3 */
    double *qtens;     /* N x N4 x 81 */
};

static void set_err(char *err, int errlen, const char *msg) {
    if (err && errlen > 0) {
        strncpy(err, msg, (size_t)errlen - 1);
        err[errlen - 1] = 0;
    }
}

/* Linear index of (b, n1..nD) in the sorted site list: basis slowest, last
 * lattice dimension fastest (lattice.jl:29-33 sorts product(1:nb, 1:L1, ...)). */
static int64_t arith_index(const orc_lattice *l, int b, const int *n) {
    int64_t lin = b - 1;
    for (int d = 0; d < l->D; d++) lin = lin * l->shape[d] + (n[d] - 1);
    return lin;
}

/* findfirst(x -> x == (bj, new_ind...), indices) (lattice.jl:196,228,273). */
static int64_t lookup(const orc_lattice *l, int literal, int bj, const int *n) {
    if (literal) {
        for (int64_t i = 0; i < l->N; i++) {
            const int32_t *t = l->idx + i * (1 + l->D);
            if (t[0] != bj) continue;
            int same = 1;
            for (int d = 0; d < l->D; d++)
                if (t[1 + d] != n[d]) { same = 0; break; }
            if (same) return i;
        }
        return -1;
    }
    if (bj < 1 || bj > l->nb) return -1;
    for (int d = 0; d < l->D; d++)
        if (n[d] < 1 || n[d] > l->shape[d]) return -1;
    return arith_index(l, bj, n);
}

/* BC(index, offset) (lattice.jl:101-109): periodic wraps with Julia's floored
 * mod, open leaves the coordinate out of range so the lookup fails. */
static void bc_apply(const orc_lattice *l, const int32_t *index, const int *off, int *out) {
    for (int d = 0; d < l->D; d++) {
        int v = index[1 + d] + off[d];
        if (l->periodic) {
            int m = (v - 1) % l->shape[d];
            if (m < 0) m += l->shape[d];
            v = m + 1;
        }
        out[d] = v;
    }
}

static void transpose9(const double *m, double *t) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) t[a * 3 + b] = m[b * 3 + a];
}

/* permutedims of a 3x3x3 tensor by a transposition of index 0 with index p. */
static void perm3(const double *J, int p, double *out) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++) {
                int i[3] = {a, b, c}, j[3] = {a, b, c};
                j[0] = i[p];
                j[p] = i[0];
                out[(a * 3 + b) * 3 + c] = J[(j[0] * 3 + j[1]) * 3 + j[2]];
            }
}

static void perm4(const double *J, int p, double *out) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++)
                for (int e = 0; e < 3; e++) {
                    int i[4] = {a, b, c, e}, j[4] = {a, b, c, e};
                    j[0] = i[p];
                    j[p] = i[0];
                    out[((a * 3 + b) * 3 + c) * 3 + e] = J[((j[0] * 3 + j[1]) * 3 + j[2]) * 3 + j[3]];
                }
}

orc_lattice *orc_lattice_new(const orc_desc *d, int literal, char *err, int errlen) {
    if (!d || d->dim < 1 || d->dim > 3) {
        set_err(err, errlen, "dim must be 1, 2 or 3");
        return NULL;
    }
    orc_lattice *l = (orc_lattice *)calloc(1, sizeof(orc_lattice));
    l->D = d->dim;
    /* Lattice() adds a basis site at the origin when the unit cell has none
     * (lattice.jl:68-70). */
    l->nb = d->n_basis > 0 ? d->n_basis : 1;
    l->periodic = d->periodic ? 1 : 0;
    l->S = d->spin_length;
    l->cells = 1;
    for (int k = 0; k < l->D; k++) {
        if (d->shape[k] < 1) {
            set_err(err, errlen, "shape entries must be >= 1");
            free(l);
            return NULL;
        }
        l->shape[k] = d->shape[k];
        l->cells *= d->shape[k];
    }
    l->N = l->cells * l->nb;
    l->N2 = d->n_bilinear;
    l->N3 = d->n_cubic;
    l->N4 = d->n_quartic;
    int64_t N = l->N;
    int D = l->D;

    /* basis indices of every term must name an existing basis site */
    for (int t = 0; t < d->n_bilinear * 2; t++)
        if (d->bilinear_basis[t] < 1 || d->bilinear_basis[t] > l->nb) goto bad_basis;
    for (int t = 0; t < d->n_cubic * 3; t++)
        if (d->cubic_basis[t] < 1 || d->cubic_basis[t] > l->nb) goto bad_basis;
    for (int t = 0; t < d->n_quartic * 4; t++)
        if (d->quartic_basis[t] < 1 || d->quartic_basis[t] > l->nb) goto bad_basis;

    l->idx = (int32_t *)malloc(sizeof(int32_t) * (size_t)(N * (1 + D)));
    for (int64_t i = 0; i < N; i++) {
        int64_t r = i;
        int32_t *t = l->idx + i * (1 + D);
        for (int k = D - 1; k >= 0; k--) {
            t[1 + k] = (int32_t)(r % l->shape[k]) + 1;
            r /= l->shape[k];
        }
        t[0] = (int32_t)r + 1;
    }

    /* Zeeman field and onsite matrix per basis, with the reference's
     * assignment rule (lattice.jl:120-140): for basis i that appears in the
     * index list, column f_indices[i] receives the i-th entry.  Where that
     * rule would index past the list (a BoundsError in Julia) or leave a
     * column unassigned (Julia would read uninitialised memory) the
     * description is rejected. */
    double *fcol = (double *)calloc((size_t)l->nb * 3, sizeof(double));
    double *ocol = (double *)calloc((size_t)l->nb * 9, sizeof(double));
    char *fset = (char *)calloc((size_t)l->nb, 1), *oset = (char *)calloc((size_t)l->nb, 1);
    for (int i = 1; i <= l->nb; i++) {
        int in_f = 0, in_o = 0;
        for (int k = 0; k < d->n_field; k++) in_f |= d->field_basis[k] == i;
        for (int k = 0; k < d->n_onsite; k++) in_o |= d->onsite_basis[k] == i;
        if (!in_f) {
            memset(fcol + (i - 1) * 3, 0, 3 * sizeof(double));
            fset[i - 1] = 1;
        } else {
            if (i > d->n_field) goto bad_field;
            int col = d->field_basis[i - 1];
            memcpy(fcol + (col - 1) * 3, d->field_vec + (i - 1) * 3, 3 * sizeof(double));
            fset[col - 1] = 1;
        }
        if (!in_o) {
            memset(ocol + (i - 1) * 9, 0, 9 * sizeof(double));
            oset[i - 1] = 1;
        } else {
            if (i > d->n_onsite) goto bad_field;
            int col = d->onsite_basis[i - 1];
            memcpy(ocol + (col - 1) * 9, d->onsite_mat + (i - 1) * 9, 9 * sizeof(double));
            oset[col - 1] = 1;
        }
    }
    for (int i = 0; i < l->nb; i++)
        if (!fset[i] || !oset[i]) goto bad_field;

    l->field = (double *)malloc(sizeof(double) * (size_t)N * 3);
    l->onsite = (double *)malloc(sizeof(double) * (size_t)N * 9);
    l->bsites = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N * l->N2 + 1));
    l->bmats = (double *)calloc((size_t)(N * l->N2 * 9 + 1), sizeof(double));
    l->csites = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N * l->N3 * 2 + 1));
    l->ctens = (double *)calloc((size_t)(N * l->N3 * 27 + 1), sizeof(double));
    l->qsites = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N * l->N4 * 3 + 1));
    l->qtens = (double *)calloc((size_t)(N * l->N4 * 81 + 1), sizeof(double));

    int nj[3], nk[3], nl[3];
    int jo[3], ko[3], lo[3];
    for (int64_t i = 0; i < N; i++) {
        const int32_t *index = l->idx + i * (1 + D);
        int b = index[0];
        memcpy(l->field + i * 3, fcol + (b - 1) * 3, 3 * sizeof(double));
        memcpy(l->onsite + i * 9, ocol + (b - 1) * 9, 9 * sizeof(double));

        /* bilinear (lattice.jl:176-204) */
        for (int t = 0; t < l->N2; t++) {
            int b1 = d->bilinear_basis[2 * t], b2 = d->bilinear_basis[2 * t + 1];
            const double *M = d->bilinear_mat + 9 * t;
            int64_t *slot = l->bsites + i * l->N2 + t;
            double *mat = l->bmats + (i * l->N2 + t) * 9;
            *slot = -1;
            if (b != b1 && b != b2) continue;
            int bj, sign;
            double Mt[9];
            const double *Muse = M;
            if (b1 == b2) {
                bj = b;
                sign = 1;
            } else if (b1 == b) {
                bj = b2;
                sign = 1;
            } else {
                bj = b1;
                sign = -1;
                transpose9(M, Mt);
                Muse = Mt;
            }
            for (int k = 0; k < D; k++) jo[k] = sign * d->bilinear_offset[t * D + k];
            bc_apply(l, index, jo, nj);
            int64_t j = lookup(l, literal, bj, nj);
            if (j >= 0) {
                *slot = j;
                memcpy(mat, Muse, 9 * sizeof(double));
            }
        }
        /* cubic (lattice.jl:209-237) */
        for (int t = 0; t < l->N3; t++) {
            int b1 = d->cubic_basis[3 * t], b2 = d->cubic_basis[3 * t + 1], b3 = d->cubic_basis[3 * t + 2];
            const double *J = d->cubic_tensor + 27 * t;
            int64_t *slot = l->csites + (i * l->N3 + t) * 2;
            double *ten = l->ctens + (i * l->N3 + t) * 27;
            slot[0] = slot[1] = -1;
            if (b != b1 && b != b2 && b != b3) continue;
            int bj, bk, p = 0;
            for (int k = 0; k < D; k++) {
                jo[k] = d->cubic_offset[t * 2 * D + k];
                ko[k] = d->cubic_offset[t * 2 * D + D + k];
            }
            if (b1 == b) {
                bj = b2;
                bk = b3;
            } else if (b2 == b) {
                bj = b1;
                bk = b3;
                for (int k = 0; k < D; k++) {
                    ko[k] = ko[k] - jo[k];
                    jo[k] = -jo[k];
                }
                p = 1;
            } else {
                bj = b2;
                bk = b1;
                for (int k = 0; k < D; k++) {
                    jo[k] = jo[k] - ko[k];
                    ko[k] = -ko[k];
                }
                p = 2;
            }
            bc_apply(l, index, jo, nj);
            bc_apply(l, index, ko, nk);
            int64_t j = lookup(l, literal, bj, nj), k2 = lookup(l, literal, bk, nk);
            if (j >= 0 && k2 >= 0) {
                slot[0] = j;
                slot[1] = k2;
                if (p == 0) memcpy(ten, J, 27 * sizeof(double));
                else perm3(J, p, ten);
            }
        }
        /* quartic (lattice.jl:243-283) */
        for (int t = 0; t < l->N4; t++) {
            const int32_t *bb = d->quartic_basis + 4 * t;
            const double *J = d->quartic_tensor + 81 * t;
            int64_t *slot = l->qsites + (i * l->N4 + t) * 3;
            double *ten = l->qtens + (i * l->N4 + t) * 81;
            slot[0] = slot[1] = slot[2] = -1;
            if (b != bb[0] && b != bb[1] && b != bb[2] && b != bb[3]) continue;
            int bj, bk, bl, p = 0;
            for (int k = 0; k < D; k++) {
                jo[k] = d->quartic_offset[t * 3 * D + k];
                ko[k] = d->quartic_offset[t * 3 * D + D + k];
                lo[k] = d->quartic_offset[t * 3 * D + 2 * D + k];
            }
            if (bb[0] == b) {
                bj = bb[1];
                bk = bb[2];
                bl = bb[3];
            } else if (bb[1] == b) {
                bj = bb[0];
                bk = bb[2];
                bl = bb[3];
                for (int k = 0; k < D; k++) {
                    jo[k] = -jo[k];
                    ko[k] = ko[k] + jo[k];
                    lo[k] = lo[k] + jo[k];
                }
                p = 1;
            } else if (bb[2] == b) {
                bj = bb[1];
                bk = bb[0];
                bl = bb[3];
                for (int k = 0; k < D; k++) {
                    ko[k] = -ko[k];
                    lo[k] = lo[k] + ko[k];
                    jo[k] = jo[k] + ko[k];
                }
                p = 2;
            } else {
                bj = bb[1];
                bk = bb[2];
                bl = bb[0];
                for (int k = 0; k < D; k++) {
                    lo[k] = -lo[k];
                    jo[k] = jo[k] + lo[k];
                    ko[k] = ko[k] + lo[k];
                }
                p = 3;
            }
            bc_apply(l, index, jo, nj);
            bc_apply(l, index, ko, nk);
            bc_apply(l, index, lo, nl);
            int64_t j = lookup(l, literal, bj, nj), k2 = lookup(l, literal, bk, nk),
                    l2 = lookup(l, literal, bl, nl);
            if (j >= 0 && k2 >= 0 && l2 >= 0) {
                slot[0] = j;
                slot[1] = k2;
                slot[2] = l2;
                if (p == 0) memcpy(ten, J, 81 * sizeof(double));
                else perm4(J, p, ten);
            }
        }
    }
    free(fcol);
    free(ocol);
    free(fset);
    free(oset);
    return l;

bad_field:
    set_err(err, errlen,
            "field/onsite assignment: the reference's per-basis rule (lattice.jl:128-139) "
            "indexes past the term list or leaves a basis unassigned; add one entry per "
            "basis in basis order");
    free(fcol);
    free(ocol);
    free(fset);
    free(oset);
    orc_lattice_free(l);
    return NULL;
bad_basis:
    set_err(err, errlen, "term names a basis index outside 1..n_basis");
    free(l);
    return NULL;
}

void orc_lattice_free(orc_lattice *l) {
    if (!l) return;
    free(l->idx);
    free(l->field);
    free(l->onsite);
    free(l->bsites);
    free(l->bmats);
    free(l->csites);
    free(l->ctens);
    free(l->qsites);
    free(l->qtens);
    free(l);
}

int64_t orc_n_sites(const orc_lattice *l) { return l->N; }

void orc_term_counts(const orc_lattice *l, int32_t out[3]) {
    out[0] = l->N2;
    out[1] = l->N3;
    out[2] = l->N4;
}

void orc_export_tables(const orc_lattice *l, int64_t *bs, double *bm, int64_t *cs, double *ct,
                       int64_t *qs, double *qt, double *field, double *onsite) {
    int64_t N = l->N;
    if (bs)
        for (int64_t k = 0; k < N * l->N2; k++) bs[k] = l->bsites[k] + 1;
    if (bm) memcpy(bm, l->bmats, sizeof(double) * (size_t)(N * l->N2 * 9));
    if (cs)
        for (int64_t k = 0; k < N * l->N3 * 2; k++) cs[k] = l->csites[k] + 1;
    if (ct) memcpy(ct, l->ctens, sizeof(double) * (size_t)(N * l->N3 * 27));
    if (qs)
        for (int64_t k = 0; k < N * l->N4 * 3; k++) qs[k] = l->qsites[k] + 1;
    if (qt) memcpy(qt, l->qtens, sizeof(double) * (size_t)(N * l->N4 * 81));
    if (field) memcpy(field, l->field, sizeof(double) * (size_t)N * 3);
    if (onsite) memcpy(onsite, l->onsite, sizeof(double) * (size_t)N * 9);
}

/* ---------------------------------------------------------------- Hamiltonian */

/* get_local_field (hamiltonian.jl:3-67).  The cubic/quartic contractions
 * follow Einsum.jl 0.4.1's expansion of `@einsum Hx += C[1,a,b]*sj[a]*sk[b]`:
 * a fresh accumulator, the first summed index innermost, then added to Hx. */
void orc_local_field(const orc_lattice *l, const double *sp, int64_t i, double H[3]) {
    const double *o = l->onsite + i * 9;
    const double *s = sp + 3 * i;
    double Hx = 0.0, Hy = 0.0, Hz = 0.0;
    Hx += 2 * (o[0] * s[0] + o[1] * s[1] + o[2] * s[2]);
    Hy += 2 * (o[3] * s[0] + o[4] * s[1] + o[5] * s[2]);
    Hz += 2 * (o[6] * s[0] + o[7] * s[1] + o[8] * s[2]);
    for (int n = 0; n < l->N2; n++) {
        int64_t j = l->bsites[i * l->N2 + n];
        if (j < 0) continue;
        const double *J = l->bmats + (i * l->N2 + n) * 9;
        const double *t = sp + 3 * j;
        Hx += J[0] * t[0] + J[1] * t[1] + J[2] * t[2];
        Hy += J[3] * t[0] + J[4] * t[1] + J[5] * t[2];
        Hz += J[6] * t[0] + J[7] * t[1] + J[8] * t[2];
    }
    for (int n = 0; n < l->N3; n++) {
        const int64_t *jk = l->csites + (i * l->N3 + n) * 2;
        if (jk[0] < 0) continue;
        const double *C = l->ctens + (i * l->N3 + n) * 27;
        const double *sj = sp + 3 * jk[0], *sk = sp + 3 * jk[1];
        double *Hc[3] = {&Hx, &Hy, &Hz};
        for (int a0 = 0; a0 < 3; a0++) {
            double acc = 0.0;
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++) acc += C[(a0 * 3 + a) * 3 + b] * sj[a] * sk[b];
            *Hc[a0] += acc;
        }
    }
    for (int n = 0; n < l->N4; n++) {
        const int64_t *jkl = l->qsites + (i * l->N4 + n) * 3;
        if (jkl[0] < 0) continue;
        const double *R = l->qtens + (i * l->N4 + n) * 81;
        const double *sj = sp + 3 * jkl[0], *sk = sp + 3 * jkl[1], *sl = sp + 3 * jkl[2];
        double *Hc[3] = {&Hx, &Hy, &Hz};
        for (int a0 = 0; a0 < 3; a0++) {
            double acc = 0.0;
            for (int c = 0; c < 3; c++)
                for (int b = 0; b < 3; b++)
                    for (int a = 0; a < 3; a++)
                        acc += R[((a0 * 3 + a) * 3 + b) * 3 + c] * sj[a] * sk[b] * sl[c];
            *Hc[a0] += acc;
        }
    }
    const double *h = l->field + i * 3;
    H[0] = Hx - h[0];
    H[1] = Hy - h[1];
    H[2] = Hz - h[2];
}

static double bilinear_term(const double *s, const double *J, const double *t) {
    return s[0] * (J[0] * t[0] + J[1] * t[1] + J[2] * t[2]) +
           s[1] * (J[3] * t[0] + J[4] * t[1] + J[5] * t[2]) +
           s[2] * (J[6] * t[0] + J[7] * t[1] + J[8] * t[2]);
}

static double cubic_term(const double *C, const double *s, const double *sj, const double *sk) {
    double acc = 0.0;
    for (int c = 0; c < 3; c++)
        for (int b = 0; b < 3; b++)
            for (int a = 0; a < 3; a++) acc += C[(a * 3 + b) * 3 + c] * s[a] * sj[b] * sk[c];
    return acc;
}

static double quartic_term(const double *R, const double *s, const double *sj, const double *sk,
                           const double *sl) {
    double acc = 0.0;
    for (int e = 0; e < 3; e++)
        for (int c = 0; c < 3; c++)
            for (int b = 0; b < 3; b++)
                for (int a = 0; a < 3; a++)
                    acc += R[((a * 3 + b) * 3 + c) * 3 + e] * s[a] * sj[b] * sk[c] * sl[e];
    return acc;
}

/* energy(lattice, point) (hamiltonian.jl:139-196). */
double orc_site_energy(const orc_lattice *l, const double *sp, int64_t i) {
    const double *o = l->onsite + i * 9;
    const double *s = sp + 3 * i;
    double E = 0.0;
    E += s[0] * (o[0] * s[0] + o[1] * s[1] + o[2] * s[2]) +
         s[1] * (o[3] * s[0] + o[4] * s[1] + o[5] * s[2]) +
         s[2] * (o[6] * s[0] + o[7] * s[1] + o[8] * s[2]);
    for (int n = 0; n < l->N2; n++) {
        int64_t j = l->bsites[i * l->N2 + n];
        if (j < 0) continue;
        E += bilinear_term(s, l->bmats + (i * l->N2 + n) * 9, sp + 3 * j);
    }
    for (int n = 0; n < l->N3; n++) {
        const int64_t *jk = l->csites + (i * l->N3 + n) * 2;
        if (jk[0] < 0) continue;
        double acc = cubic_term(l->ctens + (i * l->N3 + n) * 27, s, sp + 3 * jk[0], sp + 3 * jk[1]);
        E += acc;
    }
    for (int n = 0; n < l->N4; n++) {
        const int64_t *jkl = l->qsites + (i * l->N4 + n) * 3;
        if (jkl[0] < 0) continue;
        double acc = quartic_term(l->qtens + (i * l->N4 + n) * 81, s, sp + 3 * jkl[0],
                                  sp + 3 * jkl[1], sp + 3 * jkl[2]);
        E += acc;
    }
    const double *h = l->field + i * 3;
    return E - (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]);
}

/* total_energy (hamiltonian.jl:70-132). */
double orc_total_energy(const orc_lattice *l, const double *sp) {
    double Eb = 0.0, Ec = 0.0, Eq = 0.0, Ez = 0.0, Eo = 0.0;
    for (int64_t i = 0; i < l->N; i++) {
        const double *o = l->onsite + i * 9;
        const double *h = l->field + i * 3;
        const double *s = sp + 3 * i;
        Ez -= (s[0] * h[0] + s[1] * h[1] + s[2] * h[2]);
        Eo += s[0] * (o[0] * s[0] + o[1] * s[1] + o[2] * s[2]) +
              s[1] * (o[3] * s[0] + o[4] * s[1] + o[5] * s[2]) +
              s[2] * (o[6] * s[0] + o[7] * s[1] + o[8] * s[2]);
        for (int n = 0; n < l->N2; n++) {
            int64_t j = l->bsites[i * l->N2 + n];
            if (j < 0) continue;
            Eb += bilinear_term(s, l->bmats + (i * l->N2 + n) * 9, sp + 3 * j);
        }
        for (int n = 0; n < l->N3; n++) {
            const int64_t *jk = l->csites + (i * l->N3 + n) * 2;
            if (jk[0] < 0) continue;
            Ec += cubic_term(l->ctens + (i * l->N3 + n) * 27, s, sp + 3 * jk[0], sp + 3 * jk[1]);
        }
        for (int n = 0; n < l->N4; n++) {
            const int64_t *jkl = l->qsites + (i * l->N4 + n) * 3;
            if (jkl[0] < 0) continue;
            Eq += quartic_term(l->qtens + (i * l->N4 + n) * 81, s, sp + 3 * jkl[0],
                               sp + 3 * jkl[1], sp + 3 * jkl[2]);
        }
    }
    return Eb / 2 + Ec / 3 + Eq / 4 + Ez + Eo;
}

/* LinearAlgebra.norm of a 3-tuple: generic_norm2 sums squares in order when
 * no rescaling is needed. */
static double norm3(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

/* get_magnetization (observables.jl:12-18). */
double orc_magnetization(const orc_lattice *l, const double *sp) {
    double mx = 0.0, my = 0.0, mz = 0.0;
    for (int64_t i = 0; i < l->N; i++) {
        mx = mx + sp[3 * i];
        my = my + sp[3 * i + 1];
        mz = mz + sp[3 * i + 2];
    }
    return norm3(mx, my, mz);
}

/* compute_equal_time_correlations (spin_correlations.jl:6-43).  The
 * reference forms the row phase = exp.(-im * k' * pos) (:21) and the products
 * phase * x (:22-24): exp(-i t) = cos t - i sin t with t = k.r_i summed over
 * the dimensions in order, then Suv rows (:32-40) divided by lat.size (:42). */
void orc_structure_factor(const double *sp, int64_t N, const double *pos, int dim, const double *ks, int64_t n_k,
                          double *Suv) {
    for (int64_t n = 0; n < n_k; n++) {
        double re[3] = {0.0, 0.0, 0.0}, im[3] = {0.0, 0.0, 0.0};
        for (int64_t i = 0; i < N; i++) {
            double t = 0.0;
            for (int d = 0; d < dim; d++) t = t + ks[n * dim + d] * pos[i * dim + d];
            const double c = cos(t), s = -sin(t);
            for (int a = 0; a < 3; a++) {
                re[a] = re[a] + c * sp[3 * i + a];
                im[a] = im[a] + s * sp[3 * i + a];
            }
        }
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) /* Re((re_a + i im_a)(re_b - i im_b)) */
                Suv[n * 9 + 3 * a + b] = (re[a] * re[b] + im[a] * im[b]) / (double)N;
    }
}

/* ------------------------------------------------------------------ updates */

static const double TWO_PI = 6.283185307179586; /* 2.0 * pi in Float64 */

/* random_spin_orientation (lattice.jl:306-311). */
void orc_random_spin_orientation(double S, double u_phi, double u_z, double out[3]) {
    double phi = TWO_PI * u_phi;
    double z = 2.0 * u_z - 1.0;
    double r = sqrt(1.0 - z * z);
    out[0] = S * (r * cos(phi));
    out[1] = S * (r * sin(phi));
    out[2] = S * z;
}

/* gaussian_move (metropolis.jl:84-87). */
void orc_gaussian_move(double S, const double s[3], double sigma, double u_phi, double u_z,
                       double out[3]) {
    double r[3];
    orc_random_spin_orientation(S, u_phi, u_z, r);
    double x = s[0] + sigma * r[0], y = s[1] + sigma * r[1], z = s[2] + sigma * r[2];
    double n = norm3(x, y, z);
    out[0] = x / n * S;
    out[1] = y / n * S;
    out[2] = z / n * S;
}

/* calculate_energy_diff! (metropolis.jl:94-110). */
double orc_energy_diff(const orc_lattice *l, double *sp, int64_t i, const double ns[3]) {
    double E_old = orc_site_energy(l, sp, i);
    sp[3 * i] = ns[0];
    sp[3 * i + 1] = ns[1];
    sp[3 * i + 2] = ns[2];
    double E_new = orc_site_energy(l, sp, i);
    return E_new - E_old;
}

/* One proposal with its uniforms; returns 1 if accepted (metropolis.jl:65-82). */
static int propose(const orc_lattice *l, double *sp, int64_t i, double T, int kind,
                   double sigma, double u_phi, double u_z, double (*u_acc)(void *), void *ctx) {
    double old[3] = {sp[3 * i], sp[3 * i + 1], sp[3 * i + 2]};
    double ns[3];
    if (kind == ORC_UNIFORM) orc_random_spin_orientation(l->S, u_phi, u_z, ns);
    else orc_gaussian_move(l->S, old, sigma, u_phi, u_z, ns);
    double dE = orc_energy_diff(l, sp, i, ns);
    int accept = (dE < 0) ? 1 : (u_acc(ctx) < exp(-(dE) / T));
    if (!accept) {
        sp[3 * i] = old[0];
        sp[3 * i + 1] = old[1];
        sp[3 * i + 2] = old[2];
    }
    return accept;
}

/* sigma adaptation of metropolis_adaptive! (metropolis.jl:124-126). */
static double adapt_sigma(double sigma, double accepted, double n) {
    double a = accepted / n;
    double one_minus = 1 - a;
    double f = 0.5 / (one_minus > 0.05 ? one_minus : 0.05);
    double s = sigma * f;
    if (s < 0.0) s = 0.0;
    if (s > 100) s = 100;
    return s;
}

typedef struct {
    const double *u;
    int64_t p;
} replay_acc;
static double replay_u(void *c) {
    replay_acc *r = (replay_acc *)c;
    return r->u[r->p];
}

int64_t orc_metropolis_replay(const orc_lattice *l, double *sp, double T, int kind,
                              double *sigma, int64_t n, const int64_t *site,
                              const double *u_phi, const double *u_z, const double *u_acc,
                              uint8_t *accepted) {
    int64_t acc = 0;
    double sig = sigma ? *sigma : 60.0;
    replay_acc ra = {u_acc, 0};
    for (int64_t p = 0; p < n; p++) {
        ra.p = p;
        int a = propose(l, sp, site[p], T, kind, sig, u_phi[p], u_z[p], replay_u, &ra);
        if (accepted) accepted[p] = (uint8_t)a;
        acc += a;
    }
    if (kind == ORC_ADAPTIVE && sigma) *sigma = adapt_sigma(sig, (double)acc, (double)n);
    return acc;
}

/* ------------------------------------------------- constrained Metropolis */

double orc_constraint_value(const orc_lattice *l, const double *sp, const orc_constraint *k) {
    double V0 = 0.0, V1 = 0.0, V2 = 0.0;
    for (int64_t i = 0; i < l->N; i++) {
        double w = k->w ? k->w[i] : 1.0;
        V0 = V0 + w * sp[3 * i];
        V1 = V1 + w * sp[3 * i + 1];
        V2 = V2 + w * sp[3 * i + 2];
    }
    double vv = V0 * V0 + V1 * V1 + V2 * V2;
    return k->g[0] * V0 + k->g[1] * V1 + k->g[2] * V2 + k->q * vv + k->p * sqrt(vv) + k->c0;
}

/* One constrained proposal (metropolis.jl:42-55 / 161-174). */
static int propose_constrained(const orc_lattice *l, double *sp, int64_t i, double T, int cone, double sigma,
                               double u_phi, double u_z, double u_acc, const orc_constraint *k, double *lambda) {
    double old[3] = {sp[3 * i], sp[3 * i + 1], sp[3 * i + 2]};
    double ns[3];
    if (!cone) orc_random_spin_orientation(l->S, u_phi, u_z, ns);
    else orc_gaussian_move(l->S, old, sigma, u_phi, u_z, ns);
    double dE = orc_energy_diff(l, sp, i, ns);
    double c = orc_constraint_value(l, sp, k);
    double new_lambda = *lambda - k->weight * c;
    double x = dE - (new_lambda * c);
    int accept = x < 0 ? 1 : (u_acc < exp(-(x) / T));
    if (!accept) {
        sp[3 * i] = old[0];
        sp[3 * i + 1] = old[1];
        sp[3 * i + 2] = old[2];
    } else {
        *lambda = new_lambda;
    }
    return accept;
}

/* sigma rule of metropolis_constraint_adaptive! (metropolis.jl:175-177). */
static double adapt_sigma_constraint(double sigma, double sigma0, double accepted, double n) {
    double a = accepted / n;
    double f = 0.5 / (1 - a);
    return a < 0.5 ? sigma * f : sigma0;
}

int64_t orc_metropolis_constraint_replay(const orc_lattice *l, double *sp, double T, int cone, double *sigma,
                                         double sigma0, const orc_constraint *k, double *lambda, int64_t n,
                                         const int64_t *site, const double *u_phi, const double *u_z,
                                         const double *u_acc, uint8_t *accepted) {
    int64_t acc = 0;
    double sig = sigma ? *sigma : 60.0;
    for (int64_t p = 0; p < n; p++) {
        int a = propose_constrained(l, sp, site[p], T, cone, sig, u_phi[p], u_z[p], u_acc[p], k, lambda);
        if (accepted) accepted[p] = (uint8_t)a;
        acc += a;
    }
    if (cone && sigma) *sigma = adapt_sigma_constraint(sig, sigma0, (double)acc, (double)n);
    return acc;
}

/* overrelaxation! body (monte_carlo.jl:127-138). */
static void overrelax_site(const orc_lattice *l, double *sp, int64_t i) {
    double *s = sp + 3 * i;
    double H[3];
    orc_local_field(l, sp, i, H);
    if (H[0] == 0.0 && H[1] == 0.0 && H[2] == 0.0) return;
    double proj = 2.0 * (s[0] * H[0] + s[1] * H[1] + s[2] * H[2]) / (H[0] * H[0] + H[1] * H[1] + H[2] * H[2]);
    double nx = -s[0] + proj * H[0], ny = -s[1] + proj * H[1], nz = -s[2] + proj * H[2];
    s[0] = nx;
    s[1] = ny;
    s[2] = nz;
}

/* deterministic_updates! body (monte_carlo.jl:205-210). */
static void deterministic_site(const orc_lattice *l, double *sp, int64_t i) {
    double H[3];
    orc_local_field(l, sp, i, H);
    if (H[0] == 0.0 && H[1] == 0.0 && H[2] == 0.0) return;
    double n = norm3(H[0], H[1], H[2]);
    sp[3 * i] = -H[0] / n * l->S;
    sp[3 * i + 1] = -H[1] / n * l->S;
    sp[3 * i + 2] = -H[2] / n * l->S;
}

void orc_overrelax_order(const orc_lattice *l, double *sp, const int64_t *order, int64_t n) {
    for (int64_t k = 0; k < n; k++)
        if (order[k] >= 0) overrelax_site(l, sp, order[k]);
}

void orc_deterministic_order(const orc_lattice *l, double *sp, const int64_t *order, int64_t n) {
    for (int64_t k = 0; k < n; k++)
        if (order[k] >= 0) deterministic_site(l, sp, order[k]);
}

void orc_overrelax_sweep(const orc_lattice *l, double *sp) {
    for (int64_t i = 0; i < l->N; i++) overrelax_site(l, sp, i);
}

/* -------------------------------------------------------------------- Philox */

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Stream purposes in counter word 3; identical in the GPU kernels. */
enum { PURPOSE_METRO_A = 1, PURPOSE_METRO_B = 2, PURPOSE_SWAP = 3, PURPOSE_INIT = 4, PURPOSE_CONS_A = 5,
       PURPOSE_CONS_B = 6 };

static double u24(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }
static double u53(uint32_t a, uint32_t b) {
    uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)m * (1.0 / 9007199254740992.0);
}

typedef struct {
    uint32_t key[2];
    uint32_t d, chain, sweep;
    int bits;
    double u_acc24;
} colour_acc;
static double colour_u(void *c) {
    colour_acc *a = (colour_acc *)c;
    if (a->bits == 24) return a->u_acc24;
    uint32_t ctr[4] = {a->d, a->sweep, a->chain, PURPOSE_METRO_B}, w[4];
    orc_philox4x32_10(ctr, a->key, w);
    return u53(w[0], w[1]);
}

int64_t orc_metropolis_colour_sweep(const orc_lattice *l, double *sp, double T, int kind,
                                    double *sigma, const int64_t *order, int64_t n_order,
                                    uint64_t seed, uint32_t chain, uint32_t sweep, int bits) {
    colour_acc ca;
    ca.key[0] = (uint32_t)seed;
    ca.key[1] = (uint32_t)(seed >> 32);
    ca.chain = chain;
    ca.sweep = sweep;
    ca.bits = bits;
    double sig = sigma ? *sigma : 60.0;
    int64_t acc = 0;
    for (int64_t d = 0; d < n_order; d++) {
        if (order[d] < 0) continue;
        uint32_t ctr[4] = {(uint32_t)d, sweep, chain, PURPOSE_METRO_A}, w[4];
        orc_philox4x32_10(ctr, ca.key, w);
        double up, uz;
        if (bits == 24) {
            up = u24(w[0]);
            uz = u24(w[1]);
            ca.u_acc24 = u24(w[2]);
        } else {
            up = u53(w[0], w[1]);
            uz = u53(w[2], w[3]);
        }
        ca.d = (uint32_t)d;
        acc += propose(l, sp, order[d], T, kind, sig, up, uz, colour_u, &ca);
    }
    if (kind == ORC_ADAPTIVE && sigma) *sigma = adapt_sigma(sig, (double)acc, (double)l->N);
    return acc;
}

int64_t orc_metropolis_constraint_sweep(const orc_lattice *l, double *sp, double T, int cone, double *sigma,
                                        double sigma0, const orc_constraint *k, double *lambda, uint64_t seed,
                                        uint32_t chain, uint32_t sweep) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    double sig = sigma ? *sigma : 60.0;
    int64_t acc = 0;
    for (int64_t q = 0; q < l->N; q++) {
        uint32_t ca[4] = {(uint32_t)q, sweep, chain, PURPOSE_CONS_A}, cb[4] = {(uint32_t)q, sweep, chain, PURPOSE_CONS_B};
        uint32_t A[4], B[4];
        orc_philox4x32_10(ca, key, A);
        orc_philox4x32_10(cb, key, B);
        int64_t i = (int64_t)(((uint64_t)A[0] * (uint64_t)l->N) >> 32);
        acc += propose_constrained(l, sp, i, T, cone, sig, u53(B[0], B[1]), u53(B[2], B[3]), u53(A[2], A[3]), k,
                                   lambda);
    }
    if (cone && sigma) *sigma = adapt_sigma_constraint(sig, sigma0, (double)acc, (double)l->N);
    return acc;
}

void orc_random_spins(const orc_lattice *l, double *sp, uint64_t seed, uint32_t chain) {
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int64_t i = 0; i < l->N; i++) {
        uint32_t ctr[4] = {(uint32_t)i, 0u, chain, PURPOSE_INIT}, w[4];
        orc_philox4x32_10(ctr, key, w);
        orc_random_spin_orientation(l->S, u53(w[0], w[1]), u53(w[2], w[3]), sp + 3 * i);
    }
}

/* ------------------------------------------------------- reference drivers */

static uint64_t splitmix64(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void orc_rng_seed(orc_rng *r, uint64_t seed) {
    uint64_t x = seed;
    for (int k = 0; k < 4; k++) r->s[k] = splitmix64(&x);
}

static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t xoshiro_next(orc_rng *r) {
    uint64_t *s = r->s;
    uint64_t result = rotl(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
}

double orc_rng_uniform(orc_rng *r) { return (double)(xoshiro_next(r) >> 11) * (1.0 / 9007199254740992.0); }

static int64_t rng_site(orc_rng *r, int64_t N) {
    /* rand(1:N): unbiased by rejection */
    uint64_t n = (uint64_t)N, lim = UINT64_MAX - UINT64_MAX % n;
    uint64_t x;
    do x = xoshiro_next(r);
    while (x >= lim);
    return (int64_t)(x % n);
}

static double rng_u(void *c) { return orc_rng_uniform((orc_rng *)c); }

double orc_metropolis_sweep_ref(const orc_lattice *l, double *sp, double T, int kind,
                                double *sigma, orc_rng *r) {
    double acc = 0.0;
    double sig = sigma ? *sigma : 60.0;
    for (int64_t sweep = 0; sweep < l->N; sweep++) {
        int64_t point = rng_site(r, l->N);
        double up = orc_rng_uniform(r);
        double uz = orc_rng_uniform(r);
        acc += propose(l, sp, point, T, kind, sig, up, uz, rng_u, r);
    }
    if (kind == ORC_ADAPTIVE && sigma) *sigma = adapt_sigma(sig, acc, (double)l->N);
    return acc;
}

void orc_deterministic_ref(const orc_lattice *l, double *sp, int64_t t_det, orc_rng *r) {
    for (int64_t sweeps = 1; sweeps < t_det; sweeps++) deterministic_site(l, sp, rng_site(r, l->N));
}

double orc_simulated_annealing(const orc_lattice *l, double *sp, const double *temps,
                               int32_t n_temps, int64_t t_therm, int32_t or_rate, int kind,
                               double sigma0, orc_rng *r) {
    double total = 0.0;
    for (int32_t k = 0; k < n_temps; k++) {
        double T = temps[k];
        double sigma = sigma0;
        for (int64_t t = 1; t < t_therm; t++) {
            if (or_rate != 0) {
                orc_overrelax_sweep(l, sp);
                if (t % or_rate == 0) total += orc_metropolis_sweep_ref(l, sp, T, kind, &sigma, r);
            } else {
                total += orc_metropolis_sweep_ref(l, sp, T, kind, &sigma, r);
            }
        }
    }
    return total;
}

/* ------------------------------------------------------- parallel tempering */

typedef struct {
    const orc_lattice *lat;
    const orc_pt_params *p;
    double **spins;
    const double *T;
    double *E, *sigma, *acc;
    orc_rng *rng;
    double *probe_E, *probe_M;
    int64_t n_probe_cap;
    int32_t R;
    int64_t from, to; /* inclusive sweep range of this segment */
    int to_is_swap;   /* the probe of `to` waits for the exchange */
    int32_t next_slot;
    pthread_mutex_t mu;
} pt_shared;

static int64_t probe_index(const orc_pt_params *p, int64_t sweep) {
    if (sweep < p->t_thermalization || p->probe_rate <= 0 || sweep % p->probe_rate) return -1;
    /* probes happen at sweeps >= t_therm that are multiples of probe_rate */
    int64_t first = ((p->t_thermalization + p->probe_rate - 1) / p->probe_rate) * p->probe_rate;
    return (sweep - first) / p->probe_rate;
}

static void pt_probe(pt_shared *s, int32_t r, int64_t sweep) {
    int64_t k = probe_index(s->p, sweep);
    if (k < 0 || k >= s->n_probe_cap) return;
    if (s->probe_E) s->probe_E[k * s->R + r] = s->E[r];
    if (s->probe_M) s->probe_M[k * s->R + r] = orc_magnetization(s->lat, s->spins[r]);
}

/* monte_carlo.jl:295-377 for one slot over sweeps [from, to]. */
static void pt_segment(pt_shared *s, int32_t r) {
    const orc_pt_params *p = s->p;
    int64_t dosweep = p->overrelaxation_rate == 0 ? 1 : p->overrelaxation_rate;
    for (int64_t sweep = s->from; sweep <= s->to; sweep++) {
        if (p->overrelaxation_rate != 0) orc_overrelax_sweep(s->lat, s->spins[r]);
        if (sweep % dosweep == 0) {
            s->acc[r] += orc_metropolis_sweep_ref(s->lat, s->spins[r], s->T[r], p->kind,
                                                  &s->sigma[r], &s->rng[r]);
            s->E[r] = orc_total_energy(s->lat, s->spins[r]);
        }
        if (!(sweep == s->to && s->to_is_swap)) pt_probe(s, r, sweep);
    }
}

static void *pt_worker(void *arg) {
    pt_shared *s = (pt_shared *)arg;
    for (;;) {
        pthread_mutex_lock(&s->mu);
        int32_t r = s->next_slot++;
        pthread_mutex_unlock(&s->mu);
        if (r >= s->R) break;
        pt_segment(s, r);
    }
    return NULL;
}

int64_t orc_parallel_tempering(const orc_lattice *lat, double **spins, const double *T,
                               int32_t R, const orc_pt_params *p, double *accepted,
                               double *exchanged, double *probe_E, double *probe_M,
                               int64_t n_probe_cap) {
    pt_shared s;
    memset(&s, 0, sizeof(s));
    s.lat = lat;
    s.p = p;
    s.spins = spins;
    s.T = T;
    s.R = R;
    s.probe_E = probe_E;
    s.probe_M = probe_M;
    s.n_probe_cap = n_probe_cap;
    s.E = (double *)calloc((size_t)R, sizeof(double));
    s.sigma = (double *)calloc((size_t)R, sizeof(double));
    s.acc = (double *)calloc((size_t)R, sizeof(double));
    double *exch = (double *)calloc((size_t)R, sizeof(double));
    s.rng = (orc_rng *)calloc((size_t)R, sizeof(orc_rng));
    pthread_mutex_init(&s.mu, NULL);
    for (int32_t r = 0; r < R; r++) {
        s.E[r] = orc_total_energy(lat, spins[r]); /* monte_carlo.jl:265 */
        s.sigma[r] = p->sigma0;
        orc_rng_seed(&s.rng[r], p->seed + 0x1000193ull * (uint64_t)(r + 1));
    }
    int exchange = (R > 1 && p->swap_rate > 0);
    int64_t total = p->t_thermalization + p->t_measurement;
    int64_t dosweep = p->overrelaxation_rate == 0 ? 1 : p->overrelaxation_rate;
    int nthr = p->n_threads > 0 ? p->n_threads : 1;
    if (nthr > R) nthr = R;
    pthread_t *th = (pthread_t *)calloc((size_t)nthr, sizeof(pthread_t));

    int64_t from = 0;
    while (from < total) {
        /* next exchange point: a sweep that is a multiple of dosweep and swap_rate */
        int64_t to = total - 1;
        int to_is_swap = 0;
        if (exchange) {
            for (int64_t sw = from; sw < total; sw++)
                if (sw % dosweep == 0 && sw % p->swap_rate == 0) {
                    to = sw;
                    to_is_swap = 1;
                    break;
                }
        }
        s.from = from;
        s.to = to;
        s.to_is_swap = to_is_swap;
        s.next_slot = 0;
        for (int t = 0; t < nthr; t++) pthread_create(&th[t], NULL, pt_worker, &s);
        for (int t = 0; t < nthr; t++) pthread_join(th[t], NULL);
        if (to_is_swap) {
            /* monte_carlo.jl:308-349: pairs alternate between (even, even+1)
             * and (even-1, even); the even rank decides with its own RNG. */
            int64_t phase = (to / p->swap_rate) % 2;
            for (int32_t a = (int32_t)phase; a + 1 < R; a += 2) {
                int32_t b = a + 1;
                int32_t ev = (a % 2 == 0) ? a : b, od = (ev == a) ? b : a;
                double delta_beta = (1 / T[od] - 1 / T[ev]);
                double delta_E = (s.E[od] - s.E[ev]);
                double x = exp(delta_beta * delta_E);
                int acc = orc_rng_uniform(&s.rng[ev]) < (x < 1.0 ? x : 1.0);
                if (acc) {
                    double *tmp = spins[a];
                    spins[a] = spins[b];
                    spins[b] = tmp;
                    double e = s.E[a];
                    s.E[a] = s.E[b];
                    s.E[b] = e;
                    exch[a] += 1;
                    exch[b] += 1;
                }
            }
            for (int32_t r = 0; r < R; r++) pt_probe(&s, r, to);
        }
        from = to + 1;
    }
    int64_t n_probes = 0;
    for (int64_t sw = 0; sw < total; sw++)
        if (probe_index(p, sw) >= 0) n_probes++;
    if (accepted) memcpy(accepted, s.acc, sizeof(double) * (size_t)R);
    if (exchanged) memcpy(exchanged, exch, sizeof(double) * (size_t)R);
    pthread_mutex_destroy(&s.mu);
    free(th);
    free(s.E);
    free(s.sigma);
    free(s.acc);
    free(exch);
    free(s.rng);
    return n_probes;
}
