// plan.hpp -- host-side flattening of a lattice description into the device
// tables of the sweep kernels: per-basis term slots, deduplicated coupling
// tensors, the interaction-hypergraph colouring and the colour-major device
// order.  Shared by the C-ABI (api.cu) and the table exports.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/csmc.h"

namespace csmc {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// Owned copy of a csmc_lattice_desc.
struct Desc {
    int D = 0, nb = 1, periodic = 1;
    int shape[3] = {1, 1, 1};
    double S = 0.5;
    std::vector<int32_t> field_b, onsite_b, bil_b, cub_b, qua_b;
    std::vector<double> field_v, onsite_m, bil_m, cub_t, qua_t;
    std::vector<int32_t> bil_o, cub_o, qua_o;
    int n_bil() const { return (int)bil_b.size() / 2; }
    int n_cub() const { return (int)cub_b.size() / 3; }
    int n_qua() const { return (int)qua_b.size() / 4; }
};

Desc copy_desc(const csmc_lattice_desc *d);

// A term as seen from a site of basis b: the reference's role resolution
// (lattice.jl:176-283) gives partner bases, offsets relative to the site's
// cell and the permuted coupling tensor.
struct Slot {
    int term = 0;          // index into the unit cell's term list
    int arity = 2;         // 2 bilinear, 3 cubic, 4 quartic
    int pb[3] = {0, 0, 0}; // partner bases (1-based)
    int off[3][3] = {{0}}; // partner offsets
    std::vector<double> coef; // 9, 27 or 81 doubles
    int coef_id = 0;       // index into the deduplicated table of that arity
    bool self = false;     // bilinear slot whose partner is the site itself
};

struct Plan {
    Desc desc;
    int64_t cells = 1, N = 0;
    int N2 = 0, N3 = 0, N4 = 0;
    // per basis (0-based b): field, onsite, slots of each arity in term order
    std::vector<std::array<double, 3>> field_b;
    std::vector<std::array<double, 9>> onsite_b;
    std::vector<std::vector<Slot>> s2, s3, s4;
    // self-loop bilinear matrices folded per basis: H += P s, E += s.P.s
    std::vector<std::array<double, 9>> self_b;
    int W2 = 0, W3 = 0, W4 = 0; // non-self slot widths of the device tables
    // deduplicated coefficients; id 0 of each table is all zeros
    std::vector<double> mats, cubs, quas;
    // isotropic forms of the cubic and quartic tensors, per tensor id:
    // cub_iso {1, kappa} when C[a,b,c] = kappa eps_abc, quartic
    // qua_iso {1, q1, q2, q3} when R[a,b,c,d] = q1 d_ab d_cd + q2 d_ac d_bd +
    // q3 d_ad d_bc (exactly); {0, ...} otherwise
    std::vector<double> cub_iso, qua_iso;
    // mat_iso {1, J} when a bilinear matrix is J times the identity
    std::vector<double> mat_iso;
    // colouring and device order
    int n_colours = 0;
    std::vector<int32_t> colour_of;  // reference order
    std::vector<int64_t> col_start;  // n_colours + 1 (last = sentinel block)
    std::vector<int64_t> col_count;
    int64_t Np = 0, sentinel = 0;
    std::vector<int64_t> dev2ref, ref2dev;
    // device tables (device order, non-self slots; absent -> sentinel)
    std::vector<uint32_t> p2, p3, p4; // [W][k][Np]
    std::vector<uint8_t> pat;         // basis of each device site; nb for padding
    std::vector<int32_t> c2, c3, c4;  // [(nb+1) * W] coefficient ids per pattern
    std::string colouring_method;

    // partner of reference site i through (pb, off) or -1 (open boundary)
    int64_t partner(int64_t i, int pb, const int *off) const;
    int basis_of(int64_t i) const { return (int)(i / cells); }
};

// Build everything; throws csmc::Error.
Plan make_plan(const csmc_lattice_desc *d);

// Layout of one replica split over the CTAs of a thread-block cluster: rank
// k holds part k of every colour class (parts of `part[c]` sites, a multiple
// of 32, in device order), laid out class by class in its shared memory and
// followed by a 32-site block of zeros (its sentinel).  Partners are encoded
// ((owner rank - reading rank) mod ranks) << 14 | owner-local index, so a
// partner in the reading rank's own part has the top two bits clear.
constexpr int CLUSTER_MAX = 4;
struct ClusterLayout {
    int ranks = 1;
    int64_t Npl = 0;                     // local length per rank (incl. sentinel block)
    std::vector<int64_t> part;           // [colour] sites per part
    std::vector<int64_t> loc_start;      // [rank][colour]
    std::vector<int64_t> loc_count;      // [rank][colour]
    std::vector<int64_t> src_start;      // [rank][colour] device index of the part's first site
    // [rank][W2][Npl]: (owner rank - reading rank mod ranks) << 14 | owner-local index
    std::vector<uint16_t> q2;
    // the same for the cubic and quartic partners: [rank][W3 * 2][Npl],
    // [rank][W4 * 3][Npl]; and the basis of each local site, [rank][Npl]
    // (padding: the padding pattern nb)
    std::vector<uint16_t> q3, q4;
    std::vector<uint8_t> pat;
};
// Throws csmc::Error if a rank would hold more than 16383 sites.
ClusterLayout make_cluster_layout(const Plan &p, int ranks);

void fill_info(const Plan &p, csmc_lattice_info *info);
void export_tables(const Plan &p, int64_t *bs, double *bm, int64_t *cs, double *ct, int64_t *qs,
                   double *qt, double *field, double *onsite);

} // namespace csmc
