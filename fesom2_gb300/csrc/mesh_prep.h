// mesh_prep.h -- host-side mesh preparation (see mesh_prep.cpp).
#pragma once
#include <string>
#include <vector>

#include "../../include/fesom_gpu.h"

namespace fesom {

struct HostTopo {
    int N2 = 0, E2 = 0, T2 = 0, nl = 0;
    std::vector<int> e_n1, e_n2, e_t1, e_t2, e_up, e_dn, e_lo, e_hi;
    std::vector<int> t_n, t_nlev, t_ulev;
    std::vector<int> n_nlev, n_ulev, n_nlevmin, n_ulevmax, n_nbl;
    std::vector<int> ne_ptr, ne_idx, nie_ptr, nie_idx;
};

bool prepare_mesh(const fesom_mesh_desc &d, HostTopo &h, std::string &err);
void find_up_downwind_triangles(const fesom_mesh_desc &d, HostTopo &h);

}  // namespace fesom
