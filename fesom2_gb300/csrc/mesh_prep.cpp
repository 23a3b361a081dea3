// mesh_prep.cpp -- host-side preparation of the mesh for the device step.
//
// Converts the reference's Fortran mesh arrays (fesom_mesh_desc) into 0-based
// topology, validates every index and level bound once (so kernels never see
// an out-of-range index), and builds:
//   * the node -> edge gather list in ascending edge order, each entry tagged
//     with the node's side of the edge (the reference scatters F to edges(1,e)
//     and -F to edges(2,e), src/oce_adv_tra_driver.F90:170-189);
//   * the node -> element list in the caller's nod_in_elem2D order;
//   * the per-edge level range [nu12, nl12] of the scatters
//     (src/oce_adv_tra_driver.F90:142-156);
//   * nboundary_lay and edge_up_dn_tri when the caller does not pass them, with
//     the algorithm of muscl_adv_init / find_up_downwind_triangles
//     (src/oce_muscl_adv.F90:92-155, 240-333).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/fesom_gpu.h"
#include "mesh_prep.h"

namespace fesom {

static bool fail(std::string &err, const std::string &msg) {
    err = msg;
    return false;
}

bool prepare_mesh(const fesom_mesh_desc &d, HostTopo &h, std::string &err) {
    if (d.nod2D <= 0 || d.elem2D <= 0 || d.edge2D <= 0 || d.nl < 3)
        return fail(err, "mesh sizes must be positive and nl >= 3");
    if (d.index_base != 0 && d.index_base != 1) return fail(err, "index_base must be 0 or 1");
    const void *req[] = {d.elem2D_nodes, d.edges, d.edge_tri, d.nod_in_elem2D_num, d.nod_in_elem2D, d.nlevels,
                         d.ulevels, d.nlevels_nod2D, d.ulevels_nod2D, d.nlevels_nod2D_min, d.ulevels_nod2D_max,
                         d.coord_nod2D, d.elem_area, d.elem_cos, d.edge_dxdy, d.edge_cross_dxdy, d.gradient_sca,
                         d.area, d.areasvol, d.hnode, d.hnode_new, d.helem, d.Z_3d_n, d.zbar_3d_n, d.zbar_n_bot};
    for (const void *p : req)
        if (!p) return fail(err, "a required mesh array is NULL");
    const int N2 = d.nod2D, E2 = d.edge2D, T2 = d.elem2D, nl = d.nl, b = d.index_base;
    h.N2 = N2; h.E2 = E2; h.T2 = T2; h.nl = nl;

    h.t_n.resize(3 * (size_t)T2);
    h.t_nlev.assign(d.nlevels, d.nlevels + T2);
    h.t_ulev.assign(d.ulevels, d.ulevels + T2);
    for (int e = 0; e < T2; e++) {
        for (int k = 0; k < 3; k++) {
            int v = d.elem2D_nodes[3 * (size_t)e + k] - b;
            if (v < 0 || v >= N2) return fail(err, "elem2D_nodes index out of range");
            h.t_n[3 * (size_t)e + k] = v;
        }
        if (h.t_ulev[e] < 1 || h.t_nlev[e] > nl || h.t_nlev[e] - h.t_ulev[e] < 1)
            return fail(err, "element levels out of range (need 1 <= ulevels < nlevels <= nl)");
    }
    h.n_nlev.assign(d.nlevels_nod2D, d.nlevels_nod2D + N2);
    h.n_ulev.assign(d.ulevels_nod2D, d.ulevels_nod2D + N2);
    h.n_nlevmin.assign(d.nlevels_nod2D_min, d.nlevels_nod2D_min + N2);
    h.n_ulevmax.assign(d.ulevels_nod2D_max, d.ulevels_nod2D_max + N2);
    for (int n = 0; n < N2; n++) {
        if (h.n_ulev[n] < 1 || h.n_nlev[n] > nl || h.n_nlev[n] - h.n_ulev[n] < 2)
            return fail(err, "node column needs at least 2 wet layers and 1 <= ulevels_nod2D < nlevels_nod2D <= nl");
    }
    // node -> element (caller's order)
    h.nie_ptr.assign(N2 + 1, 0);
    for (int n = 0; n < N2; n++) {
        int k = d.nod_in_elem2D_num[n];
        if (k < 1 || k > d.ld_nie) return fail(err, "nod_in_elem2D_num out of range");
        h.nie_ptr[n + 1] = h.nie_ptr[n] + k;
    }
    h.nie_idx.resize(h.nie_ptr[N2]);
    for (int n = 0; n < N2; n++) {
        for (int k = 0; k < d.nod_in_elem2D_num[n]; k++) {
            int el = d.nod_in_elem2D[(size_t)n * d.ld_nie + k] - b;
            if (el < 0 || el >= T2) return fail(err, "nod_in_elem2D index out of range");
            const int *tn = &h.t_n[3 * (size_t)el];
            if (tn[0] != n && tn[1] != n && tn[2] != n) return fail(err, "nod_in_elem2D lists an element not containing the node");
            h.nie_idx[h.nie_ptr[n] + k] = el;
        }
    }
    // edges
    h.e_n1.resize(E2); h.e_n2.resize(E2); h.e_t1.resize(E2); h.e_t2.resize(E2);
    h.e_lo.resize(E2); h.e_hi.resize(E2);
    for (int e = 0; e < E2; e++) {
        int n1 = d.edges[2 * (size_t)e] - b, n2 = d.edges[2 * (size_t)e + 1] - b;
        int t1 = d.edge_tri[2 * (size_t)e] - b, t2 = d.edge_tri[2 * (size_t)e + 1] - b;
        if (n1 < 0 || n1 >= N2 || n2 < 0 || n2 >= N2 || n1 == n2) return fail(err, "edges index out of range");
        if (t1 < 0 || t1 >= T2) return fail(err, "edge_tri(1,e) must be a valid element");
        if (t2 >= T2) return fail(err, "edge_tri(2,e) out of range");
        if (t2 < 0) t2 = -1;
        h.e_n1[e] = n1; h.e_n2[e] = n2; h.e_t1[e] = t1; h.e_t2[e] = t2;
        int nl1 = h.t_nlev[t1] - 1, nu1 = h.t_ulev[t1], nl2 = 0, nu2 = 0;
        if (t2 >= 0) { nl2 = h.t_nlev[t2] - 1; nu2 = h.t_ulev[t2]; }
        int nl12 = std::max(nl1, nl2), nu12 = nu1;
        if (nu2 > 0) nu12 = std::min(nu1, nu2);
        h.e_lo[e] = nu12;
        h.e_hi[e] = nl12;
        // the scatter range must lie inside both node columns
        for (int v : {n1, n2})
            if (nu12 < h.n_ulev[v] || nl12 > h.n_nlev[v] - 1) return fail(err, "edge levels exceed a node column");
        // the flux loops A..E of the reference must not overlap (true without cavities)
        int fnl12 = std::min(nl1, nl2), fnu12 = std::max(nu1, nu2);
        if (t2 >= 0 && fnl12 + 1 <= fnu12 - 1) return fail(err, "edge with disjoint wet ranges (cavity layout) is not supported");
    }
    // node -> edge, ascending edge order with side tag
    std::vector<int> cnt(N2 + 1, 0);
    for (int e = 0; e < E2; e++) { cnt[h.e_n1[e] + 1]++; cnt[h.e_n2[e] + 1]++; }
    h.ne_ptr.assign(N2 + 1, 0);
    for (int n = 0; n < N2; n++) h.ne_ptr[n + 1] = h.ne_ptr[n] + cnt[n + 1];
    h.ne_idx.resize(h.ne_ptr[N2]);
    std::vector<int> pos(h.ne_ptr.begin(), h.ne_ptr.end() - 1);
    for (int e = 0; e < E2; e++) {  // ascending e fills each list in ascending order
        h.ne_idx[pos[h.e_n1[e]]++] = e;
        h.ne_idx[pos[h.e_n2[e]]++] = ~e;
    }
    // MUSCL init arrays
    h.n_nbl.resize(N2);
    if (d.nboundary_lay) {
        h.n_nbl.assign(d.nboundary_lay, d.nboundary_lay + N2);
    } else {
        for (int n = 0; n < N2; n++) h.n_nbl[n] = nl - 1;
        for (int e = 0; e < E2; e++) {
            int n1 = h.e_n1[e], n2 = h.e_n2[e], t1 = h.e_t1[e], t2 = h.e_t2[e];
            if (t2 < 0) {
                h.n_nbl[n1] = 0;
                h.n_nbl[n2] = 0;
            } else {
                int mv = std::min(h.t_nlev[t1], h.t_nlev[t2]) - 1;
                h.n_nbl[n1] = std::min(h.n_nbl[n1], mv);
                h.n_nbl[n2] = std::min(h.n_nbl[n2], mv);
            }
        }
    }
    h.e_up.assign(E2, -1);
    h.e_dn.assign(E2, -1);
    if (d.edge_up_dn_tri) {
        for (int e = 0; e < E2; e++) {
            int u = d.edge_up_dn_tri[2 * (size_t)e] - b, w = d.edge_up_dn_tri[2 * (size_t)e + 1] - b;
            if (u >= T2 || w >= T2) return fail(err, "edge_up_dn_tri out of range");
            h.e_up[e] = u < 0 ? -1 : u;
            h.e_dn[e] = w < 0 ? -1 : w;
        }
    } else {
        find_up_downwind_triangles(d, h);
    }
    for (int e = 0; e < E2; e++) {
        for (int side = 0; side < 2; side++) {
            int tri = side == 0 ? h.e_up[e] : h.e_dn[e];
            if (tri < 0) continue;
            int node = side == 0 ? h.e_n1[e] : h.e_n2[e];
            const int *tn = &h.t_n[3 * (size_t)tri];
            if (tn[0] != node && tn[1] != node && tn[2] != node)
                return fail(err, "edge_up_dn_tri lists an element that does not contain the edge node");
        }
    }
    return true;
}

// find_up_downwind_triangles (src/oce_muscl_adv.F90:240-333): for each edge end
// node, the element around it whose corner contains the direction pointing
// away from the other end node; the last matching element in nod_in_elem2D
// order wins (the reference's `cycle` keeps scanning).
void find_up_downwind_triangles(const fesom_mesh_desc &d, HostTopo &h) {
    const double cyc = d.cyclic_length;
    const double *X = d.coord_nod2D;
    for (int e = 0; e < h.E2; e++) {
        int ed[2] = {h.e_n1[e], h.e_n2[e]};
        double x0 = X[2 * (size_t)ed[1]] - X[2 * (size_t)ed[0]];
        double x1 = X[2 * (size_t)ed[1] + 1] - X[2 * (size_t)ed[0] + 1];
        if (x0 > cyc / 2.0) x0 = x0 - cyc;
        if (x0 < -cyc / 2.0) x0 = x0 + cyc;
        for (int side = 0; side < 2; side++) {
            x0 = -x0;
            x1 = -x1;
            int node = ed[side];
            int found = -1;
            for (int k = h.nie_ptr[node]; k < h.nie_ptr[node + 1]; k++) {
                int el = h.nie_idx[k];
                const int *en = &h.t_n[3 * (size_t)el];
                int i0, i1, i2;
                if (en[0] == node) { i0 = 0; i1 = 1; i2 = 2; }
                else if (en[1] == node) { i0 = 1; i1 = 0; i2 = 2; }
                else { i0 = 2; i1 = 0; i2 = 1; }
                double b0 = X[2 * (size_t)en[i1]] - X[2 * (size_t)en[i0]];
                double b1 = X[2 * (size_t)en[i1] + 1] - X[2 * (size_t)en[i0] + 1];
                double c0 = X[2 * (size_t)en[i2]] - X[2 * (size_t)en[i0]];
                double c1 = X[2 * (size_t)en[i2] + 1] - X[2 * (size_t)en[i0] + 1];
                if (b0 > cyc / 2.0) b0 = b0 - cyc;
                if (b0 < -cyc / 2.0) b0 = b0 + cyc;
                if (c0 > cyc / 2.0) c0 = c0 - cyc;
                if (c0 < -cyc / 2.0) c0 = c0 + cyc;
                double cr = 0.0; cr += c0 * c0; cr += c1 * c1;
                double s = 0.0; s += b0 * c0; s += b1 * c1;
                double bx = s / cr;
                double by = (-(b0 * c1) + b1 * c0) / cr;
                s = 0.0; s += x0 * c0; s += x1 * c1;
                double xx = s / cr;
                double xy = (-(x0 * c1) + x1 * c0) / cr;
                double ab = std::atan2(by, bx);
                double ax = std::atan2(xy, xx);
                if ((ab > 0.0) && (ax > 0.0) && (ax < ab)) { found = el; continue; }
                if ((ab < 0.0) && (ax < 0.0) && (ax > ab)) { found = el; continue; }
                if ((ab == ax) || (ax == 0.0)) { found = el; continue; }
            }
            if (side == 0) h.e_up[e] = found;
            else h.e_dn[e] = found;
        }
    }
}

}  // namespace fesom
