// plan.cpp -- flatten a lattice description into device tables and colour
// its interaction hypergraph.
//
// The per-site term resolution restates Lattice() (lattice.jl:65-291) with
// the neighbour found by index arithmetic instead of findfirst over the sorted
// site list (lattice.jl:196,228,273): both give the same site because the
// list is sorted lexicographically by (basis, n1, ..., nD).
#include "plan.hpp"

#include <algorithm>
#include <cstring>
#include <functional>
#include <numeric>

namespace csmc {

static void require(bool ok, int code, const std::string &msg) {
    if (!ok) throw Error(code, msg);
}

Desc copy_desc(const csmc_lattice_desc *d) {
    require(d != nullptr, CSMC_ERR_INVALID, "lattice description is NULL");
    require(d->dim >= 1 && d->dim <= 3, CSMC_ERR_INVALID, "dim must be 1, 2 or 3");
    Desc o;
    o.D = d->dim;
    o.nb = d->n_basis > 0 ? d->n_basis : 1; // lattice.jl:68-70
    o.periodic = d->periodic ? 1 : 0;
    o.S = d->spin_length;
    for (int k = 0; k < o.D; k++) {
        require(d->shape[k] >= 1, CSMC_ERR_INVALID, "shape entries must be >= 1");
        o.shape[k] = d->shape[k];
    }
    auto cp_i = [](std::vector<int32_t> &v, const int32_t *p, int64_t n, const char *what) {
        require(n == 0 || p != nullptr, CSMC_ERR_INVALID, std::string(what) + " is NULL");
        v.assign(p, p + n);
    };
    auto cp_d = [](std::vector<double> &v, const double *p, int64_t n, const char *what) {
        require(n == 0 || p != nullptr, CSMC_ERR_INVALID, std::string(what) + " is NULL");
        v.assign(p, p + n);
    };
    require(d->n_field >= 0 && d->n_onsite >= 0 && d->n_bilinear >= 0 && d->n_cubic >= 0 &&
                d->n_quartic >= 0,
            CSMC_ERR_INVALID, "negative term count");
    cp_i(o.field_b, d->field_basis, d->n_field, "field_basis");
    cp_d(o.field_v, d->field_vec, 3 * (int64_t)d->n_field, "field_vec");
    cp_i(o.onsite_b, d->onsite_basis, d->n_onsite, "onsite_basis");
    cp_d(o.onsite_m, d->onsite_mat, 9 * (int64_t)d->n_onsite, "onsite_mat");
    cp_i(o.bil_b, d->bilinear_basis, 2 * (int64_t)d->n_bilinear, "bilinear_basis");
    cp_d(o.bil_m, d->bilinear_mat, 9 * (int64_t)d->n_bilinear, "bilinear_mat");
    cp_i(o.bil_o, d->bilinear_offset, (int64_t)o.D * d->n_bilinear, "bilinear_offset");
    cp_i(o.cub_b, d->cubic_basis, 3 * (int64_t)d->n_cubic, "cubic_basis");
    cp_d(o.cub_t, d->cubic_tensor, 27 * (int64_t)d->n_cubic, "cubic_tensor");
    cp_i(o.cub_o, d->cubic_offset, 2 * (int64_t)o.D * d->n_cubic, "cubic_offset");
    cp_i(o.qua_b, d->quartic_basis, 4 * (int64_t)d->n_quartic, "quartic_basis");
    cp_d(o.qua_t, d->quartic_tensor, 81 * (int64_t)d->n_quartic, "quartic_tensor");
    cp_i(o.qua_o, d->quartic_offset, 3 * (int64_t)o.D * d->n_quartic, "quartic_offset");
    auto chk = [&](const std::vector<int32_t> &v) {
        for (int32_t b : v)
            require(b >= 1 && b <= o.nb, CSMC_ERR_INVALID,
                    "term names basis " + std::to_string(b) + " outside 1.." + std::to_string(o.nb));
    };
    chk(o.bil_b);
    chk(o.cub_b);
    chk(o.qua_b);
    for (int32_t b : o.field_b) require(b >= 1, CSMC_ERR_INVALID, "field basis must be >= 1");
    for (int32_t b : o.onsite_b) require(b >= 1, CSMC_ERR_INVALID, "onsite basis must be >= 1");
    return o;
}

int64_t Plan::partner(int64_t i, int pb, const int *off) const {
    // site (b, n) of reference index i; BC(index, offset) (lattice.jl:101-109)
    int64_t r = i % cells;
    int n[3] = {0, 0, 0};
    for (int k = desc.D - 1; k >= 0; k--) {
        n[k] = (int)(r % desc.shape[k]);
        r /= desc.shape[k];
    }
    int64_t lin = pb - 1;
    for (int k = 0; k < desc.D; k++) {
        int64_t v = (int64_t)n[k] + off[k];
        int64_t L = desc.shape[k];
        if (desc.periodic) {
            v %= L;
            if (v < 0) v += L;
        } else if (v < 0 || v >= L) {
            return -1;
        }
        lin = lin * L + v;
    }
    return lin;
}

// permutedims by the transposition (0 p) of a 3^k tensor, k = 3 or 4.
static std::vector<double> transpose_first(const std::vector<double> &J, int k, int p) {
    std::vector<double> out(J.size());
    int n = (int)J.size();
    for (int lin = 0; lin < n; lin++) {
        int idx[4], r = lin;
        for (int q = k - 1; q >= 0; q--) {
            idx[q] = r % 3;
            r /= 3;
        }
        int src[4];
        for (int q = 0; q < k; q++) src[q] = idx[q];
        src[0] = idx[p];
        src[p] = idx[0];
        int s = 0;
        for (int q = 0; q < k; q++) s = s * 3 + src[q];
        out[lin] = J[s];
    }
    return out;
}

static void resolve_slots(Plan &P) {
    const Desc &d = P.desc;
    const int D = d.D, nb = d.nb;
    P.s2.assign(nb, {});
    P.s3.assign(nb, {});
    P.s4.assign(nb, {});
    for (int b = 1; b <= nb; b++) {
        // bilinear (lattice.jl:176-204)
        for (int t = 0; t < d.n_bil(); t++) {
            int b1 = d.bil_b[2 * t], b2 = d.bil_b[2 * t + 1];
            if (b != b1 && b != b2) continue;
            Slot s;
            s.term = t;
            s.arity = 2;
            const double *M = &d.bil_m[9 * t];
            int sign = 1;
            if (b1 == b2) {
                s.pb[0] = b;
            } else if (b1 == b) {
                s.pb[0] = b2;
            } else {
                s.pb[0] = b1;
                sign = -1;
            }
            s.coef.assign(M, M + 9);
            if (sign < 0) // transposeJ (interaction_matrix.jl:27-31)
                for (int a = 0; a < 3; a++)
                    for (int c = 0; c < 3; c++) s.coef[a * 3 + c] = M[c * 3 + a];
            for (int k = 0; k < D; k++) s.off[0][k] = sign * d.bil_o[t * D + k];
            P.s2[b - 1].push_back(s);
        }
        // cubic (lattice.jl:209-237)
        for (int t = 0; t < d.n_cub(); t++) {
            const int32_t *bb = &d.cub_b[3 * t];
            if (b != bb[0] && b != bb[1] && b != bb[2]) continue;
            Slot s;
            s.term = t;
            s.arity = 3;
            int jo[3] = {0, 0, 0}, ko[3] = {0, 0, 0};
            for (int k = 0; k < D; k++) {
                jo[k] = d.cub_o[t * 2 * D + k];
                ko[k] = d.cub_o[t * 2 * D + D + k];
            }
            std::vector<double> J(&d.cub_t[27 * t], &d.cub_t[27 * t] + 27);
            if (bb[0] == b) {
                s.pb[0] = bb[1];
                s.pb[1] = bb[2];
                s.coef = J;
            } else if (bb[1] == b) {
                s.pb[0] = bb[0];
                s.pb[1] = bb[2];
                for (int k = 0; k < D; k++) {
                    ko[k] = ko[k] - jo[k];
                    jo[k] = -jo[k];
                }
                s.coef = transpose_first(J, 3, 1);
            } else {
                s.pb[0] = bb[1];
                s.pb[1] = bb[0];
                for (int k = 0; k < D; k++) {
                    jo[k] = jo[k] - ko[k];
                    ko[k] = -ko[k];
                }
                s.coef = transpose_first(J, 3, 2);
            }
            for (int k = 0; k < D; k++) {
                s.off[0][k] = jo[k];
                s.off[1][k] = ko[k];
            }
            P.s3[b - 1].push_back(s);
        }
        // quartic (lattice.jl:243-283)
        for (int t = 0; t < d.n_qua(); t++) {
            const int32_t *bb = &d.qua_b[4 * t];
            if (b != bb[0] && b != bb[1] && b != bb[2] && b != bb[3]) continue;
            Slot s;
            s.term = t;
            s.arity = 4;
            int jo[3] = {0, 0, 0}, ko[3] = {0, 0, 0}, lo[3] = {0, 0, 0};
            for (int k = 0; k < D; k++) {
                jo[k] = d.qua_o[t * 3 * D + k];
                ko[k] = d.qua_o[t * 3 * D + D + k];
                lo[k] = d.qua_o[t * 3 * D + 2 * D + k];
            }
            std::vector<double> J(&d.qua_t[81 * t], &d.qua_t[81 * t] + 81);
            if (bb[0] == b) {
                s.pb[0] = bb[1];
                s.pb[1] = bb[2];
                s.pb[2] = bb[3];
                s.coef = J;
            } else if (bb[1] == b) {
                s.pb[0] = bb[0];
                s.pb[1] = bb[2];
                s.pb[2] = bb[3];
                for (int k = 0; k < D; k++) {
                    jo[k] = -jo[k];
                    ko[k] = ko[k] + jo[k];
                    lo[k] = lo[k] + jo[k];
                }
                s.coef = transpose_first(J, 4, 1);
            } else if (bb[2] == b) {
                s.pb[0] = bb[1];
                s.pb[1] = bb[0];
                s.pb[2] = bb[3];
                for (int k = 0; k < D; k++) {
                    ko[k] = -ko[k];
                    lo[k] = lo[k] + ko[k];
                    jo[k] = jo[k] + ko[k];
                }
                s.coef = transpose_first(J, 4, 2);
            } else {
                s.pb[0] = bb[1];
                s.pb[1] = bb[2];
                s.pb[2] = bb[0];
                for (int k = 0; k < D; k++) {
                    lo[k] = -lo[k];
                    jo[k] = jo[k] + lo[k];
                    ko[k] = ko[k] + lo[k];
                }
                s.coef = transpose_first(J, 4, 3);
            }
            for (int k = 0; k < D; k++) {
                s.off[0][k] = jo[k];
                s.off[1][k] = ko[k];
                s.off[2][k] = lo[k];
            }
            P.s4[b - 1].push_back(s);
        }
    }
}

// Is the k-th partner of a slot the site itself?  Translation invariance makes
// this a property of (basis, slot): same basis and an offset that maps a cell
// to itself.
static bool partner_is_self(const Plan &P, int b, const Slot &s, int k) {
    if (s.pb[k] != b) return false;
    for (int q = 0; q < P.desc.D; q++) {
        int o = s.off[k][q], L = P.desc.shape[q];
        if (P.desc.periodic ? (o % L != 0) : (o != 0)) return false;
    }
    return true;
}

// Zeeman field and onsite matrix per basis with the reference's assignment
// rule (lattice.jl:120-140): for basis i present in the index list, column
// f_indices[i] gets the i-th entry.  Cases where Julia would throw a
// BoundsError or read an unassigned column are rejected.
static void assign_per_basis(Plan &P) {
    const Desc &d = P.desc;
    int nb = d.nb;
    auto run = [&](const std::vector<int32_t> &idx, const std::vector<double> &val, int w,
                   std::vector<double> &out, const char *what) {
        out.assign((size_t)nb * w, 0.0);
        std::vector<char> set(nb, 0);
        int n = (int)idx.size();
        for (int i = 1; i <= nb; i++) {
            bool in = std::find(idx.begin(), idx.end(), i) != idx.end();
            if (!in) {
                set[i - 1] = 1;
                continue;
            }
            require(i <= n, CSMC_ERR_INVALID,
                    std::string(what) +
                        ": basis " + std::to_string(i) +
                        " appears in the list but the reference indexes its entry " +
                        std::to_string(i) + " (lattice.jl:128-139); add one entry per basis "
                        "in basis order");
            int col = idx[i - 1];
            require(col >= 1 && col <= nb, CSMC_ERR_INVALID,
                    std::string(what) + " names basis " + std::to_string(col) + " outside 1..nb");
            std::copy(&val[(size_t)(i - 1) * w], &val[(size_t)(i - 1) * w] + w,
                      &out[(size_t)(col - 1) * w]);
            set[col - 1] = 1;
        }
        for (int b = 0; b < nb; b++)
            require(set[b], CSMC_ERR_INVALID,
                    std::string(what) + ": the reference's per-basis rule (lattice.jl:128-139) "
                                        "leaves basis " +
                        std::to_string(b + 1) + " unassigned");
    };
    std::vector<double> f, o;
    run(d.field_b, d.field_v, 3, f, "field");
    run(d.onsite_b, d.onsite_m, 9, o, "onsite");
    P.field_b.resize(nb);
    P.onsite_b.resize(nb);
    for (int b = 0; b < nb; b++) {
        for (int k = 0; k < 3; k++) P.field_b[b][k] = f[b * 3 + k];
        for (int k = 0; k < 9; k++) P.onsite_b[b][k] = o[b * 9 + k];
    }
}

// The isotropic forms of the deduplicated coupling tensors (see
// Plan::cub_iso): J times the identity for the bilinear matrices; the only
// rotation-invariant rank-3 tensor is eps_abc, the rank-4 ones are the three
// pairings of delta products.  A tensor is tagged only if it equals the form
// entry by entry; the kernels then evaluate J s_j, kappa (s_j x s_k) and
// q1 s_j (s_k.s_l) + q2 s_k (s_j.s_l) + q3 s_l (s_j.s_k) instead of the dense
// contraction.
static void classify_isotropic(Plan &P) {
    auto eps = [](int a, int b, int c) {
        if (a == b || b == c || a == c) return 0;
        return ((a + 1) % 3 == b) ? 1 : -1; // (0,1,2) and its cyclic shifts: +1
    };
    const size_t nm = P.mats.size() / 9, nc = P.cubs.size() / 27, nq = P.quas.size() / 81;
    P.mat_iso.assign(2 * nm, 0.0);
    for (size_t t = 0; t < nm; t++) {
        const double *M = &P.mats[9 * t];
        bool ok = true;
        for (int k = 0; k < 9; k++)
            if (M[k] != (k % 4 == 0 ? M[0] : 0.0)) ok = false;
        if (ok) {
            P.mat_iso[2 * t] = 1.0;
            P.mat_iso[2 * t + 1] = M[0];
        }
    }
    P.cub_iso.assign(2 * nc, 0.0);
    for (size_t t = 0; t < nc; t++) {
        const double *C = &P.cubs[27 * t];
        const double k = C[(0 * 3 + 1) * 3 + 2];
        bool ok = true;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                for (int c = 0; c < 3; c++) {
                    const int e = eps(a, b, c);
                    const double want = e == 0 ? 0.0 : (e > 0 ? k : -k);
                    if (C[(a * 3 + b) * 3 + c] != want) ok = false;
                }
        if (ok) {
            P.cub_iso[2 * t] = 1.0;
            P.cub_iso[2 * t + 1] = k;
        }
    }
    P.qua_iso.assign(4 * nq, 0.0);
    for (size_t t = 0; t < nq; t++) {
        const double *Q = &P.quas[81 * t];
        auto at = [&](int a, int b, int c, int d) { return Q[((a * 3 + b) * 3 + c) * 3 + d]; };
        const double q1 = at(0, 0, 1, 1), q2 = at(0, 1, 0, 1), q3 = at(0, 1, 1, 0);
        bool ok = true;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                for (int c = 0; c < 3; c++)
                    for (int d = 0; d < 3; d++) {
                        double want = 0.0;
                        if (a == b && c == d) want += q1;
                        if (a == c && b == d) want += q2;
                        if (a == d && b == c) want += q3;
                        if (at(a, b, c, d) != want) ok = false;
                    }
        if (ok) {
            P.qua_iso[4 * t] = 1.0;
            P.qua_iso[4 * t + 1] = q1;
            P.qua_iso[4 * t + 2] = q2;
            P.qua_iso[4 * t + 3] = q3;
        }
    }
}

static int dedup(std::vector<double> &table, int width, const std::vector<double> &c) {
    int n = (int)(table.size() / width);
    for (int k = 0; k < n; k++)
        if (std::memcmp(&table[(size_t)k * width], c.data(), sizeof(double) * width) == 0) return k;
    table.insert(table.end(), c.begin(), c.end());
    return n;
}

// ------------------------------------------------------------------ colouring

// Read-partners of every site (non-self), for the conflict graph.
template <class F> static void for_partners(const Plan &P, int64_t i, F &&f) {
    int b = P.basis_of(i);
    auto visit = [&](const std::vector<Slot> &v) {
        for (const Slot &s : v) {
            if (s.self) continue;
            for (int k = 0; k < s.arity - 1; k++) {
                int64_t p = P.partner(i, s.pb[k], s.off[k]);
                if (p >= 0 && p != i) f(p);
            }
        }
    };
    visit(P.s2[b]);
    visit(P.s3[b]);
    visit(P.s4[b]);
}

// Exact colouring of a small graph by backtracking in DSATUR order.
static bool colour_exact(const std::vector<std::vector<int>> &adj, int k, std::vector<int> &col,
                         long &budget) {
    int n = (int)adj.size();
    col.assign(n, -1);
    std::function<bool(int)> rec = [&](int done) -> bool {
        if (done == n) return true;
        if (--budget < 0) return false;
        int best = -1, bsat = -1, bdeg = -1;
        for (int v = 0; v < n; v++) {
            if (col[v] >= 0) continue;
            unsigned mask = 0;
            for (int u : adj[v])
                if (col[u] >= 0) mask |= 1u << col[u];
            int sat = __builtin_popcount(mask), deg = (int)adj[v].size();
            if (sat > bsat || (sat == bsat && deg > bdeg)) {
                best = v;
                bsat = sat;
                bdeg = deg;
            }
        }
        unsigned mask = 0;
        for (int u : adj[best])
            if (col[u] >= 0) mask |= 1u << col[u];
        for (int c = 0; c < k; c++) {
            if (mask & (1u << c)) continue;
            col[best] = c;
            if (rec(done + 1)) return true;
            col[best] = -1;
        }
        return false;
    };
    return rec(0);
}

// Periodic colouring: colour(b, n) = q(b, n mod p) for a small period p whose
// quotient graph has no self loop; valid on the full lattice when p divides L
// (periodic) or always (open boundaries only remove edges).
static bool quotient_colouring(const Plan &P, std::vector<int32_t> &colour, int &ncol,
                               std::string &how) {
    const Desc &d = P.desc;
    // small periods, plus each extent itself when it is small (odd tori)
    std::vector<int> cand = {1, 2, 3, 4, 6};
    for (int k = 0; k < d.D; k++)
        if (d.shape[k] <= 12 && std::find(cand.begin(), cand.end(), d.shape[k]) == cand.end())
            cand.push_back(d.shape[k]);
    std::vector<std::array<int, 3>> periods;
    for (int a : cand)
        for (int b : cand)
            for (int c : cand) {
                std::array<int, 3> p = {a, d.D > 1 ? b : 1, d.D > 2 ? c : 1};
                if (d.D < 2 && b != 1) continue;
                if (d.D < 3 && c != 1) continue;
                bool ok = true;
                for (int k = 0; k < d.D; k++) {
                    if (p[k] > d.shape[k]) ok = false;
                    if (d.periodic && d.shape[k] % p[k] != 0) ok = false;
                }
                if (ok) periods.push_back(p);
            }
    std::stable_sort(periods.begin(), periods.end(), [](const auto &x, const auto &y) {
        return x[0] * x[1] * x[2] < y[0] * y[1] * y[2];
    });
    int best = CSMC_MAX_COLOURS + 1;
    std::vector<int> best_q;
    std::array<int, 3> best_p = {1, 1, 1};
    for (const auto &p : periods) {
        int cells = p[0] * p[1] * p[2];
        int n = d.nb * cells;
        if (n > 256) continue;
        std::vector<std::vector<int>> adj(n);
        bool selfloop = false;
        for (int b = 0; b < d.nb && !selfloop; b++)
            for (int r = 0; r < cells && !selfloop; r++) {
                int rr[3] = {r / (p[1] * p[2]), (r / p[2]) % p[1], r % p[2]};
                int u = b * cells + r;
                auto visit = [&](const std::vector<Slot> &v) {
                    for (const Slot &s : v) {
                        if (s.self) continue;
                        for (int k = 0; k < s.arity - 1; k++) {
                            int q[3];
                            for (int x = 0; x < 3; x++) {
                                int o = x < d.D ? s.off[k][x] : 0;
                                q[x] = ((rr[x] + o) % p[x] + p[x]) % p[x];
                            }
                            int w = (s.pb[k] - 1) * cells + (q[0] * p[1] + q[1]) * p[2] + q[2];
                            if (w == u) {
                                selfloop = true;
                                return;
                            }
                            adj[u].push_back(w);
                            adj[w].push_back(u);
                        }
                    }
                };
                visit(P.s2[b]);
                visit(P.s3[b]);
                visit(P.s4[b]);
            }
        if (selfloop) continue;
        for (auto &a : adj) {
            std::sort(a.begin(), a.end());
            a.erase(std::unique(a.begin(), a.end()), a.end());
        }
        std::vector<int> q;
        for (int k = 1; k < best; k++) {
            long budget = 200000;
            if (colour_exact(adj, k, q, budget)) {
                best = k;
                best_q = q;
                best_p = p;
                break;
            }
        }
        if (best <= 2) break; // cannot do better than 2 with any edge
    }
    if (best > CSMC_MAX_COLOURS) return false;
    int cells = best_p[0] * best_p[1] * best_p[2];
    colour.assign(P.N, 0);
    for (int64_t i = 0; i < P.N; i++) {
        int b = P.basis_of(i);
        int64_t r = i % P.cells;
        int n[3] = {0, 0, 0};
        for (int k = d.D - 1; k >= 0; k--) {
            n[k] = (int)(r % d.shape[k]);
            r /= d.shape[k];
        }
        int q = ((n[0] % best_p[0]) * best_p[1] + (n[1] % best_p[1])) * best_p[2] + (n[2] % best_p[2]);
        colour[i] = best_q[b * cells + q];
    }
    ncol = best;
    how = "periodic quotient p=(" + std::to_string(best_p[0]) + "," + std::to_string(best_p[1]) +
          "," + std::to_string(best_p[2]) + ")";
    return true;
}

// Greedy colouring of the full conflict graph in smallest-last order.
static bool greedy_colouring(const Plan &P, std::vector<int32_t> &colour, int &ncol) {
    const int64_t N = P.N;
    std::vector<std::vector<int64_t>> adj(N);
    for (int64_t i = 0; i < N; i++)
        for_partners(P, i, [&](int64_t p) {
            adj[i].push_back(p);
            adj[p].push_back(i);
        });
    for (auto &a : adj) {
        std::sort(a.begin(), a.end());
        a.erase(std::unique(a.begin(), a.end()), a.end());
    }
    // smallest-last ordering with bucket queue
    std::vector<int64_t> deg(N);
    int64_t maxd = 0;
    for (int64_t i = 0; i < N; i++) maxd = std::max<int64_t>(maxd, deg[i] = (int64_t)adj[i].size());
    std::vector<std::vector<int64_t>> bucket(maxd + 1);
    for (int64_t i = 0; i < N; i++) bucket[deg[i]].push_back(i);
    std::vector<char> removed(N, 0);
    std::vector<int64_t> order;
    order.reserve(N);
    int64_t cur = 0;
    while ((int64_t)order.size() < N) {
        cur = std::max<int64_t>(0, cur - 1);
        while (cur <= maxd && bucket[cur].empty()) cur++;
        int64_t v = bucket[cur].back();
        bucket[cur].pop_back();
        if (removed[v] || deg[v] != cur) continue;
        removed[v] = 1;
        order.push_back(v);
        for (int64_t u : adj[v])
            if (!removed[u]) bucket[--deg[u]].push_back(u);
    }
    std::reverse(order.begin(), order.end());
    colour.assign(N, -1);
    ncol = 0;
    for (int64_t v : order) {
        unsigned long long mask = 0;
        for (int64_t u : adj[v])
            if (colour[u] >= 0 && colour[u] < 64) mask |= 1ull << colour[u];
        int c = 0;
        while (mask & (1ull << c)) c++;
        colour[v] = c;
        ncol = std::max(ncol, c + 1);
    }
    return ncol <= CSMC_MAX_COLOURS;
}

static void colour_plan(Plan &P) {
    std::vector<int32_t> cq, cg;
    int nq = 0, ng = 0;
    std::string how;
    bool okq = quotient_colouring(P, cq, nq, how);
    // the full-graph greedy only when the quotient is not already optimal
    bool tryg = !okq || nq > 2;
    int64_t work = P.N * (int64_t)(P.W2 + 2 * P.W3 + 3 * P.W4 + 1);
    bool okg = false;
    if (tryg && work < 60000000) okg = greedy_colouring(P, cg, ng);
    if (okq && (!okg || nq <= ng)) {
        P.colour_of = std::move(cq);
        P.n_colours = nq;
        P.colouring_method = how;
    } else if (okg) {
        P.colour_of = std::move(cg);
        P.n_colours = ng;
        P.colouring_method = "greedy smallest-last";
    } else {
        throw Error(CSMC_ERR_COLOURING, "no colouring with at most " +
                                            std::to_string(CSMC_MAX_COLOURS) + " colours found");
    }
    if (P.N > 0 && P.n_colours == 0) P.n_colours = 1;
    // verify: no site reads a site of its own colour
    for (int64_t i = 0; i < P.N; i++) {
        bool bad = false;
        for_partners(P, i, [&](int64_t p) { bad |= P.colour_of[p] == P.colour_of[i]; });
        if (bad)
            throw Error(CSMC_ERR_COLOURING,
                        "colouring check failed at site " + std::to_string(i) + " (" +
                            P.colouring_method + ")");
    }
}

// ------------------------------------------------------------------ plan

Plan make_plan(const csmc_lattice_desc *dd) {
    Plan P;
    P.desc = copy_desc(dd);
    const Desc &d = P.desc;
    P.cells = 1;
    for (int k = 0; k < d.D; k++) P.cells *= d.shape[k];
    P.N = P.cells * d.nb;
    require(P.N < (int64_t)1 << 31, CSMC_ERR_UNSUPPORTED, "more than 2^31 sites");
    P.N2 = d.n_bil();
    P.N3 = d.n_cub();
    P.N4 = d.n_qua();
    assign_per_basis(P);
    resolve_slots(P);

    const int nb = d.nb;
    P.self_b.assign(nb, {});
    P.mats.assign(9, 0.0);
    P.cubs.assign(27, 0.0);
    P.quas.assign(81, 0.0);
    for (int b = 0; b < nb; b++) {
        int w2 = 0;
        for (Slot &s : P.s2[b]) {
            s.self = partner_is_self(P, b + 1, s, 0);
            if (s.self) {
                for (int k = 0; k < 9; k++) P.self_b[b][k] += s.coef[k];
            } else {
                s.coef_id = dedup(P.mats, 9, s.coef);
                w2++;
            }
        }
        P.W2 = std::max(P.W2, w2);
        for (Slot &s : P.s3[b]) {
            for (int k = 0; k < 2; k++)
                require(!partner_is_self(P, b + 1, s, k), CSMC_ERR_UNSUPPORTED,
                        "a cubic term whose partner is the site itself is not supported by the "
                        "colour-sweep kernels");
            s.coef_id = dedup(P.cubs, 27, s.coef);
        }
        P.W3 = std::max(P.W3, (int)P.s3[b].size());
        for (Slot &s : P.s4[b]) {
            for (int k = 0; k < 3; k++)
                require(!partner_is_self(P, b + 1, s, k), CSMC_ERR_UNSUPPORTED,
                        "a quartic term whose partner is the site itself is not supported by the "
                        "colour-sweep kernels");
            s.coef_id = dedup(P.quas, 81, s.coef);
        }
        P.W4 = std::max(P.W4, (int)P.s4[b].size());
    }

    classify_isotropic(P);
    colour_plan(P);

    // colour-major device order, each class padded to a multiple of 32 sites,
    // then one 32-site block of zero spins whose first site is the sentinel
    const int C = P.n_colours;
    P.col_count.assign(C, 0);
    for (int64_t i = 0; i < P.N; i++) P.col_count[P.colour_of[i]]++;
    P.col_start.assign(C + 1, 0);
    int64_t pos = 0;
    for (int c = 0; c < C; c++) {
        P.col_start[c] = pos;
        pos += (P.col_count[c] + 31) / 32 * 32;
    }
    P.col_start[C] = pos;
    P.sentinel = pos;
    P.Np = pos + 32;
    require(P.Np < ((int64_t)1 << 32) - 1, CSMC_ERR_UNSUPPORTED, "lattice too large");
    P.dev2ref.assign(P.Np, -1);
    P.ref2dev.assign(P.N, -1);
    std::vector<int64_t> fill(C);
    for (int c = 0; c < C; c++) fill[c] = P.col_start[c];
    for (int64_t i = 0; i < P.N; i++) {
        int64_t dpos = fill[P.colour_of[i]]++;
        P.dev2ref[dpos] = i;
        P.ref2dev[i] = dpos;
    }

    // device tables
    const int64_t Np = P.Np;
    const uint32_t SENT = (uint32_t)P.sentinel;
    P.pat.assign(Np, (uint8_t)nb);
    require(nb < 255, CSMC_ERR_UNSUPPORTED, "more than 254 basis sites");
    P.c2.assign((size_t)(nb + 1) * std::max(P.W2, 1), 0);
    P.c3.assign((size_t)(nb + 1) * std::max(P.W3, 1), 0);
    P.c4.assign((size_t)(nb + 1) * std::max(P.W4, 1), 0);
    for (int b = 0; b < nb; b++) {
        int t = 0;
        for (const Slot &s : P.s2[b])
            if (!s.self) P.c2[(size_t)b * P.W2 + t++] = s.coef_id;
        t = 0;
        for (const Slot &s : P.s3[b]) P.c3[(size_t)b * P.W3 + t++] = s.coef_id;
        t = 0;
        for (const Slot &s : P.s4[b]) P.c4[(size_t)b * P.W4 + t++] = s.coef_id;
    }
    P.p2.assign((size_t)P.W2 * Np, SENT);
    P.p3.assign((size_t)P.W3 * 2 * Np, SENT);
    P.p4.assign((size_t)P.W4 * 3 * Np, SENT);
    for (int64_t dpos = 0; dpos < Np; dpos++) {
        int64_t i = P.dev2ref[dpos];
        if (i < 0) continue;
        int b = P.basis_of(i);
        P.pat[dpos] = (uint8_t)b;
        int t = 0;
        for (const Slot &s : P.s2[b]) {
            if (s.self) continue;
            int64_t p = P.partner(i, s.pb[0], s.off[0]);
            P.p2[(size_t)t * Np + dpos] = p >= 0 ? (uint32_t)P.ref2dev[p] : SENT;
            t++;
        }
        t = 0;
        for (const Slot &s : P.s3[b]) {
            int64_t pj = P.partner(i, s.pb[0], s.off[0]), pk = P.partner(i, s.pb[1], s.off[1]);
            bool ok = pj >= 0 && pk >= 0; // open BC zeroes the whole term (lattice.jl:230-232)
            P.p3[((size_t)t * 2 + 0) * Np + dpos] = ok ? (uint32_t)P.ref2dev[pj] : SENT;
            P.p3[((size_t)t * 2 + 1) * Np + dpos] = ok ? (uint32_t)P.ref2dev[pk] : SENT;
            t++;
        }
        t = 0;
        for (const Slot &s : P.s4[b]) {
            int64_t pj = P.partner(i, s.pb[0], s.off[0]), pk = P.partner(i, s.pb[1], s.off[1]),
                    pl = P.partner(i, s.pb[2], s.off[2]);
            bool ok = pj >= 0 && pk >= 0 && pl >= 0; // lattice.jl:276-278
            P.p4[((size_t)t * 3 + 0) * Np + dpos] = ok ? (uint32_t)P.ref2dev[pj] : SENT;
            P.p4[((size_t)t * 3 + 1) * Np + dpos] = ok ? (uint32_t)P.ref2dev[pk] : SENT;
            P.p4[((size_t)t * 3 + 2) * Np + dpos] = ok ? (uint32_t)P.ref2dev[pl] : SENT;
            t++;
        }
    }
    return P;
}

ClusterLayout make_cluster_layout(const Plan &P, int ranks) {
    require(ranks >= 1 && ranks <= CLUSTER_MAX, CSMC_ERR_INVALID, "cluster size out of range");
    ClusterLayout L;
    L.ranks = ranks;
    const int C = P.n_colours;
    L.part.assign(C, 0);
    L.loc_start.assign((size_t)ranks * C, 0);
    L.loc_count.assign((size_t)ranks * C, 0);
    L.src_start.assign((size_t)ranks * C, 0);
    std::vector<int64_t> len(ranks, 0);
    for (int c = 0; c < C; c++) {
        const int64_t n = P.col_count[c];
        L.part[c] = ((n + ranks - 1) / ranks + 31) / 32 * 32;
        for (int k = 0; k < ranks; k++) {
            const int64_t lo = std::min(n, k * L.part[c]), hi = std::min(n, (k + 1) * L.part[c]);
            L.loc_start[k * C + c] = len[k];
            L.loc_count[k * C + c] = hi - lo;
            L.src_start[k * C + c] = P.col_start[c] + lo;
            len[k] += (hi - lo + 31) / 32 * 32;
        }
    }
    int64_t mx = 0;
    for (int k = 0; k < ranks; k++) mx = std::max(mx, len[k]);
    L.Npl = mx + 32; // sentinel block at local index mx
    require(L.Npl <= 16384, CSMC_ERR_UNSUPPORTED, "a cluster rank would hold more than 16383 sites");
    const int64_t sent_local = mx;
    // device index -> (owner relative to the reader, owner-local index); the
    // reader's own sites and the sentinel have relative owner 0
    auto locate = [&](int64_t d, int reader) -> uint16_t {
        if (d == P.sentinel || d < 0) return (uint16_t)sent_local;
        int c = 0;
        while (c + 1 < C && d >= P.col_start[c + 1]) c++;
        const int64_t off = d - P.col_start[c];
        const int k = (int)(off / L.part[c]);
        const int64_t local = L.loc_start[k * C + c] + (off - k * L.part[c]);
        const int rel = (k - reader + ranks) % ranks;
        return (uint16_t)((rel << 14) | local);
    };
    const int W = std::max(P.W2, 1);
    L.q2.assign((size_t)ranks * W * L.Npl, 0);
    for (int k = 0; k < ranks; k++) {
        for (int t = 0; t < W; t++)
            for (int64_t i = 0; i < L.Npl; i++) L.q2[((size_t)k * W + t) * L.Npl + i] = (uint16_t)sent_local;
        for (int c = 0; c < C; c++)
            for (int64_t j = 0; j < L.loc_count[k * C + c]; j++) {
                const int64_t d = L.src_start[k * C + c] + j, i = L.loc_start[k * C + c] + j;
                for (int t = 0; t < P.W2; t++)
                    L.q2[((size_t)k * W + t) * L.Npl + i] = locate(P.p2[(size_t)t * P.Np + d], k);
            }
    }
    // cubic and quartic partners, and the pattern of every local site
    const int W3 = P.W3 * 2, W4 = P.W4 * 3;
    L.q3.assign((size_t)ranks * std::max(W3, 1) * L.Npl, (uint16_t)sent_local);
    L.q4.assign((size_t)ranks * std::max(W4, 1) * L.Npl, (uint16_t)sent_local);
    L.pat.assign((size_t)ranks * L.Npl, (uint8_t)P.desc.nb);
    for (int k = 0; k < ranks; k++)
        for (int c = 0; c < C; c++)
            for (int64_t j = 0; j < L.loc_count[k * C + c]; j++) {
                const int64_t d = L.src_start[k * C + c] + j, i = L.loc_start[k * C + c] + j;
                L.pat[(size_t)k * L.Npl + i] = P.pat[d];
                for (int t = 0; t < W3; t++)
                    L.q3[((size_t)k * W3 + t) * L.Npl + i] = locate(P.p3[(size_t)t * P.Np + d], k);
                for (int t = 0; t < W4; t++)
                    L.q4[((size_t)k * W4 + t) * L.Npl + i] = locate(P.p4[(size_t)t * P.Np + d], k);
            }
    return L;
}

void fill_info(const Plan &p, csmc_lattice_info *info) {
    std::memset(info, 0, sizeof(*info));
    info->n_sites = p.N;
    info->n_colours = p.n_colours;
    info->n_bilinear = p.N2;
    info->n_cubic = p.N3;
    info->n_quartic = p.N4;
    info->width_bilinear = p.W2;
    info->width_cubic = p.W3;
    info->width_quartic = p.W4;
    info->n_matrices = (int32_t)(p.mats.size() / 9);
    info->n_cubic_tensors = (int32_t)(p.cubs.size() / 27);
    info->n_quartic_tensors = (int32_t)(p.quas.size() / 81);
    info->n_isotropic_cubic = 0;
    info->n_isotropic_quartic = 0;
    for (size_t t = 0; t < p.cub_iso.size(); t += 2) info->n_isotropic_cubic += p.cub_iso[t] != 0.0;
    for (size_t t = 0; t < p.qua_iso.size(); t += 4) info->n_isotropic_quartic += p.qua_iso[t] != 0.0;
    info->padded_sites = p.Np;
}

void export_tables(const Plan &P, int64_t *bs, double *bm, int64_t *cs, double *ct, int64_t *qs,
                   double *qt, double *field, double *onsite) {
    const int64_t N = P.N;
    for (int64_t i = 0; i < N; i++) {
        int b = P.basis_of(i);
        if (field)
            for (int k = 0; k < 3; k++) field[i * 3 + k] = P.field_b[b][k];
        if (onsite)
            for (int k = 0; k < 9; k++) onsite[i * 9 + k] = P.onsite_b[b][k];
        if (bs || bm) {
            for (int t = 0; t < P.N2; t++) {
                if (bs) bs[i * P.N2 + t] = 0;
                if (bm) std::fill(bm + (i * P.N2 + t) * 9, bm + (i * P.N2 + t) * 9 + 9, 0.0);
            }
            for (const Slot &s : P.s2[b]) {
                int64_t p = P.partner(i, s.pb[0], s.off[0]);
                if (p < 0) continue;
                if (bs) bs[i * P.N2 + s.term] = p + 1;
                if (bm) std::copy(s.coef.begin(), s.coef.end(), bm + (i * P.N2 + s.term) * 9);
            }
        }
        if (cs || ct) {
            for (int t = 0; t < P.N3; t++) {
                if (cs) cs[(i * P.N3 + t) * 2] = cs[(i * P.N3 + t) * 2 + 1] = 0;
                if (ct) std::fill(ct + (i * P.N3 + t) * 27, ct + (i * P.N3 + t) * 27 + 27, 0.0);
            }
            for (const Slot &s : P.s3[b]) {
                int64_t pj = P.partner(i, s.pb[0], s.off[0]), pk = P.partner(i, s.pb[1], s.off[1]);
                if (pj < 0 || pk < 0) continue;
                if (cs) {
                    cs[(i * P.N3 + s.term) * 2] = pj + 1;
                    cs[(i * P.N3 + s.term) * 2 + 1] = pk + 1;
                }
                if (ct) std::copy(s.coef.begin(), s.coef.end(), ct + (i * P.N3 + s.term) * 27);
            }
        }
        if (qs || qt) {
            for (int t = 0; t < P.N4; t++) {
                if (qs)
                    for (int k = 0; k < 3; k++) qs[(i * P.N4 + t) * 3 + k] = 0;
                if (qt) std::fill(qt + (i * P.N4 + t) * 81, qt + (i * P.N4 + t) * 81 + 81, 0.0);
            }
            for (const Slot &s : P.s4[b]) {
                int64_t pj = P.partner(i, s.pb[0], s.off[0]), pk = P.partner(i, s.pb[1], s.off[1]),
                        pl = P.partner(i, s.pb[2], s.off[2]);
                if (pj < 0 || pk < 0 || pl < 0) continue;
                if (qs) {
                    qs[(i * P.N4 + s.term) * 3] = pj + 1;
                    qs[(i * P.N4 + s.term) * 3 + 1] = pk + 1;
                    qs[(i * P.N4 + s.term) * 3 + 2] = pl + 1;
                }
                if (qt) std::copy(s.coef.begin(), s.coef.end(), qt + (i * P.N4 + s.term) * 81);
            }
        }
    }
}

} // namespace csmc
