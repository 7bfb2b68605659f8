// Internal declarations shared by the host table builder and the engine.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "punc_gpu.h"

namespace pg {

// Host-side mesh tables.  Cell-local vertex order is ascending global vertex
// id and facet i is opposite local vertex i (the UFC convention DOLFIN uses
// after Mesh::order()).
struct HostMesh {
    int64_t nv = 0, nc = 0, ndof = 0;
    std::vector<double> coords;          // [nv][3]
    std::vector<int64_t> cell_vertices;  // [nc][4]
    std::vector<int64_t> cell_dofs;      // [nc][4]
    std::vector<double> bary;            // [nc][12]
    std::vector<double> planes;          // [nc][16]
    std::vector<int64_t> nbr;            // [nc][4], neighbour or -tag
    std::vector<double> volume;          // [nc]
    std::vector<double> dv_inv;          // [ndof]
    std::vector<int64_t> rowptr, col;    // CSR over dofs
    std::vector<double> K, M;            // eps0 * stiffness, mass
    std::vector<double> ext_facets;      // [nf][14]
    std::vector<double> obj_facets;      // [no][7]
    std::vector<int64_t> bc_kind;        // [ndof]
    int32_t n_objects = 0;               // number of object tags (max tag - 1)
    double bbox_lo[3] = {0, 0, 0}, bbox_hi[3] = {0, 0, 0};
    // Uniform bin grid over the bounding box for point location.
    int32_t nbin[3] = {1, 1, 1};
    double bin_h[3] = {1, 1, 1};
    std::vector<int64_t> bin_ptr;        // [nbins+1]
    std::vector<int32_t> bin_cells;
};

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

}  // namespace pg

struct pg_mesh {
    pg::HostMesh h;
};
