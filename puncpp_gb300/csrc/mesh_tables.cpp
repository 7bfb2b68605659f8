// Host-side mesh tables: topology, per-cell geometry, P1 matrices.
//
// This is the set-up the reference does once on the host in the
// Population<3> constructor (punc/include/punc/population.h:310-389),
// Cell<3>::init_barycentric_matrix (punc/src/population.cpp:181-240),
// element_volume (punc/src/distributor.cpp:35-69),
// Mesh::exterior_boundaries (punc/src/mesh.cpp:166-236) and the FFC-assembled
// forms of punc/ufl/Potential3D.ufl.  Every floating-point expression whose
// rounding reaches a cell index (the facet planes) or a bit-compared result
// (the barycentric matrix) is evaluated in the reference's operation order;
// this file must be compiled without floating-point contraction.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>

#include "pg_internal.h"
#include "pg_math.h"

namespace pg {

namespace {

thread_local std::string g_last_error;

// Run f(begin, end) over [0, n) on the host's cores.
template <class F>
void parallel_for(int64_t n, F f) {
    unsigned hw = std::thread::hardware_concurrency();
    int64_t nt = std::max<int64_t>(1, std::min<int64_t>(hw ? hw : 1, (n + 65535) / 65536));
    if (nt == 1) { f(0, n); return; }
    std::vector<std::thread> ts;
    int64_t chunk = (n + nt - 1) / nt;
    for (int64_t t = 0; t < nt; ++t) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        ts.emplace_back([=] { f(b, e); });
    }
    for (auto &t : ts) t.join();
}

// A facet as its three vertex ids in ascending order, with an owner slot.
struct FacetRec {
    int64_t b, c;      // second and third vertex (first is the bucket)
    int64_t slot;      // cell*4 + local facet, or boundary-list index
};

// Group facets by smallest vertex id, then sort each bucket by (b, c).
struct FacetIndex {
    std::vector<int64_t> ptr;
    std::vector<FacetRec> rec;
    void build(int64_t nv, int64_t n, const int64_t *tri /*[n][3] sorted*/,
               const int64_t *slot) {
        ptr.assign(nv + 1, 0);
        for (int64_t k = 0; k < n; ++k) ptr[tri[3 * k] + 1]++;
        for (int64_t v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
        rec.resize(n);
        std::vector<int64_t> cur(ptr.begin(), ptr.end() - 1);
        for (int64_t k = 0; k < n; ++k) {
            int64_t a = tri[3 * k];
            rec[cur[a]++] = FacetRec{tri[3 * k + 1], tri[3 * k + 2], slot[k]};
        }
        parallel_for(nv, [&](int64_t b0, int64_t e0) {
            for (int64_t v = b0; v < e0; ++v)
                std::sort(rec.begin() + ptr[v], rec.begin() + ptr[v + 1],
                          [](const FacetRec &x, const FacetRec &y) {
                              return x.b != y.b ? x.b < y.b : (x.c != y.c ? x.c < y.c : x.slot < y.slot);
                          });
        });
    }
};

inline void sort3(int64_t &a, int64_t &b, int64_t &c) {
    if (a > b) std::swap(a, b);
    if (b > c) std::swap(b, c);
    if (a > b) std::swap(a, b);
}

// Rows 0-2 of the barycentric matrix, with the expressions of
// Cell<3>::init_barycentric_matrix (punc/src/population.cpp:181-240).
void barycentric_rows(const double *p, double *A) {
    const double x1 = p[0], y1 = p[1], z1 = p[2];
    const double x2 = p[3], y2 = p[4], z2 = p[5];
    const double x3 = p[6], y3 = p[7], z3 = p[8];
    const double x4 = p[9], y4 = p[10], z4 = p[11];
    const double x13 = x1 - x3, y13 = y1 - y3, z13 = z1 - z3;
    const double x14 = x1 - x4, y14 = y1 - y4, z14 = z1 - z4;
    const double x24 = x2 - x4, y24 = y2 - y4, z24 = z2 - z4;
    const double x31 = x3 - x1, y31 = y3 - y1, z31 = z3 - z1;
    const double x32 = x3 - x2, y32 = y3 - y2, z32 = z3 - z2;
    const double x34 = x3 - x4, y34 = y3 - y4, z34 = z3 - z4;
    const double x42 = x4 - x2, y42 = y4 - y2, z42 = z4 - z2;
    const double x43 = x4 - x3, y43 = y4 - y3, z43 = z4 - z3;
    const double v1 = (x2 * (y3 * z4 - y4 * z3) + x3 * (y4 * z2 - y2 * z4) + x4 * (y2 * z3 - y3 * z2)) / 6.0;
    const double v2 = (x1 * (y4 * z3 - y3 * z4) + x3 * (y1 * z4 - y4 * z1) + x4 * (y3 * z1 - y1 * z3)) / 6.0;
    const double v3 = (x1 * (y2 * z4 - y4 * z2) + x2 * (y4 * z1 - y1 * z4) + x4 * (y1 * z2 - y2 * z1)) / 6.0;
    const double v4 = (x1 * (y3 * z2 - y2 * z3) + x2 * (y1 * z3 - y3 * z1) + x3 * (y2 * z1 - y1 * z2)) / 6.0;
    const double vol = v1 + v2 + v3 + v4;
    const double vol6 = 6 * vol;
    A[0] = v1 / vol;
    A[4] = v2 / vol;
    A[8] = v3 / vol;
    A[1] = (y42 * z32 - y32 * z42) / vol6;
    A[5] = (y31 * z43 - y34 * z13) / vol6;
    A[9] = (y24 * z14 - y14 * z24) / vol6;
    A[2] = (x32 * z42 - x42 * z32) / vol6;
    A[6] = (x43 * z31 - x13 * z34) / vol6;
    A[10] = (x14 * z24 - x24 * z14) / vol6;
    A[3] = (x42 * y32 - x32 * y42) / vol6;
    A[7] = (x31 * y43 - x34 * y13) / vol6;
    A[11] = (x24 * y14 - x14 * y24) / vol6;
}

// Outward unit normal of facet f (opposite local vertex f), restating
// DOLFIN 2019.1 TetrahedronCell::normal: n = (P2-P1) x (P3-P1) over the
// facet's ascending vertices, divided by its norm, negated when it points
// towards the opposite vertex P0.
void facet_normal(const double *p /*[4][3]*/, int f, double *n) {
    int q[3], k = 0;
    for (int i = 0; i < 4; ++i) if (i != f) q[k++] = i;
    const double *P0 = p + 3 * f, *P1 = p + 3 * q[0], *P2 = p + 3 * q[1], *P3 = p + 3 * q[2];
    const double a0 = P0[0] - P1[0], a1 = P0[1] - P1[1], a2 = P0[2] - P1[2];
    const double b0 = P2[0] - P1[0], b1 = P2[1] - P1[1], b2 = P2[2] - P1[2];
    const double c0 = P3[0] - P1[0], c1 = P3[1] - P1[1], c2 = P3[2] - P1[2];
    double nx = b1 * c2 - b2 * c1;
    double ny = b2 * c0 - b0 * c2;
    double nz = b0 * c1 - b1 * c0;
    const double len = std::sqrt(nx * nx + ny * ny + nz * nz);
    nx /= len; ny /= len; nz /= len;
    if (nx * a0 + ny * a1 + nz * a2 > 0) { nx *= -1.0; ny *= -1.0; nz *= -1.0; }
    n[0] = nx; n[1] = ny; n[2] = nz;
}

// Facet midpoint: vertex sum in ascending vertex order divided by 3
// (DOLFIN MeshEntity::midpoint).
void facet_midpoint(const double *p, int f, double *m) {
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 4; ++i) {
        if (i == f) continue;
        s[0] += p[3 * i]; s[1] += p[3 * i + 1]; s[2] += p[3 * i + 2];
    }
    m[0] = s[0] / 3.0; m[1] = s[1] / 3.0; m[2] = s[2] / 3.0;
}

// Area of facet f: half the norm of (P2-P1) x (P3-P1).
double facet_area(const double *p, int f) {
    int q[3], k = 0;
    for (int i = 0; i < 4; ++i) if (i != f) q[k++] = i;
    const double *P1 = p + 3 * q[0], *P2 = p + 3 * q[1], *P3 = p + 3 * q[2];
    const double b0 = P2[0] - P1[0], b1 = P2[1] - P1[1], b2 = P2[2] - P1[2];
    const double c0 = P3[0] - P1[0], c1 = P3[1] - P1[1], c2 = P3[2] - P1[2];
    const double nx = b1 * c2 - b2 * c1, ny = b2 * c0 - b0 * c2, nz = b0 * c1 - b1 * c0;
    return 0.5 * std::sqrt(nx * nx + ny * ny + nz * nz);
}

// |det(P1-P0, P2-P0, P3-P0)| / 6.
double tet_volume(const double *p) {
    const double a0 = p[3] - p[0], a1 = p[4] - p[1], a2 = p[5] - p[2];
    const double b0 = p[6] - p[0], b1 = p[7] - p[1], b2 = p[8] - p[2];
    const double c0 = p[9] - p[0], c1 = p[10] - p[1], c2 = p[11] - p[2];
    const double det = a0 * (b1 * c2 - b2 * c1) - a1 * (b0 * c2 - b2 * c0) + a2 * (b0 * c1 - b1 * c0);
    return std::fabs(det) / 6.0;
}

}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error_cstr() { return g_last_error.c_str(); }
int fail(int code, const std::string &msg) { set_error(msg); return code; }

int build_mesh(const pg_mesh_desc *d, double eps0, HostMesh &h) {
    if (!d || d->n_vertices <= 0 || d->n_cells <= 0 || !d->coords || !d->cells)
        return fail(PG_ERR_ARG, "pg_mesh_build: empty mesh");
    if (d->n_boundary_facets < 0 || (d->n_boundary_facets > 0 && (!d->bfacet_vertices || !d->bfacet_tags)))
        return fail(PG_ERR_ARG, "pg_mesh_build: boundary facet arrays missing");
    if (d->n_cells >= (int64_t(1) << 31) - 1)
        return fail(PG_ERR_ARG, "pg_mesh_build: more than 2^31-2 cells");
    const int64_t nv = d->n_vertices, nc = d->n_cells;
    h.nv = nv; h.nc = nc;
    h.ndof = d->vertex_to_dof ? d->n_dofs : nv;
    if (h.ndof <= 0) return fail(PG_ERR_ARG, "pg_mesh_build: n_dofs must be positive");
    h.coords.assign(d->coords, d->coords + 3 * nv);

    // Cell vertices in ascending order (UFC numbering).
    h.cell_vertices.resize(4 * nc);
    for (int64_t c = 0; c < nc; ++c) {
        int64_t v[4];
        for (int i = 0; i < 4; ++i) {
            v[i] = d->cells[4 * c + i];
            if (v[i] < 0 || v[i] >= nv) return fail(PG_ERR_MESH, "cell " + std::to_string(c) + " has an out-of-range vertex");
        }
        std::sort(v, v + 4);
        if (v[0] == v[1] || v[1] == v[2] || v[2] == v[3])
            return fail(PG_ERR_MESH, "cell " + std::to_string(c) + " repeats a vertex");
        for (int i = 0; i < 4; ++i) h.cell_vertices[4 * c + i] = v[i];
    }
    h.cell_dofs.resize(4 * nc);
    for (int64_t k = 0; k < 4 * nc; ++k) {
        int64_t v = h.cell_vertices[k];
        int64_t dof = d->vertex_to_dof ? d->vertex_to_dof[v] : v;
        if (dof < 0 || dof >= h.ndof) return fail(PG_ERR_MESH, "vertex_to_dof out of range");
        h.cell_dofs[k] = dof;
    }

    // Facet adjacency: facet i of cell c = the three other vertices.
    {
        std::vector<int64_t> tri(12 * nc), slot(4 * nc);
        for (int64_t c = 0; c < nc; ++c) {
            const int64_t *v = &h.cell_vertices[4 * c];
            for (int f = 0; f < 4; ++f) {
                int k = 0;
                for (int i = 0; i < 4; ++i) if (i != f) tri[12 * c + 3 * f + k++] = v[i];
                slot[4 * c + f] = 4 * c + f;
            }
        }
        FacetIndex fi;
        fi.build(nv, 4 * nc, tri.data(), slot.data());
        tri.clear(); tri.shrink_to_fit();
        // Boundary tags.
        const int64_t nb = d->n_boundary_facets;
        std::vector<int64_t> btri(3 * std::max<int64_t>(nb, 1)), bslot(std::max<int64_t>(nb, 1));
        for (int64_t k = 0; k < nb; ++k) {
            int64_t a = d->bfacet_vertices[3 * k], b = d->bfacet_vertices[3 * k + 1], c = d->bfacet_vertices[3 * k + 2];
            if (a < 0 || b < 0 || c < 0 || a >= nv || b >= nv || c >= nv)
                return fail(PG_ERR_MESH, "boundary facet vertex out of range");
            sort3(a, b, c);
            btri[3 * k] = a; btri[3 * k + 1] = b; btri[3 * k + 2] = c;
            bslot[k] = k;
            if (d->bfacet_tags[k] < 1) return fail(PG_ERR_MESH, "boundary facet tags must be >= 1");
        }
        FacetIndex bi;
        bi.build(nv, nb, btri.data(), bslot.data());
        h.nbr.assign(4 * nc, 0);
        int32_t max_tag = 1;
        for (int64_t a = 0; a < nv; ++a) {
            int64_t s = fi.ptr[a], e = fi.ptr[a + 1];
            int64_t k = s;
            while (k < e) {
                int64_t k2 = k + 1;
                while (k2 < e && fi.rec[k2].b == fi.rec[k].b && fi.rec[k2].c == fi.rec[k].c) ++k2;
                int64_t cnt = k2 - k;
                if (cnt == 2) {
                    int64_t s0 = fi.rec[k].slot, s1 = fi.rec[k + 1].slot;
                    h.nbr[s0] = s1 / 4;
                    h.nbr[s1] = s0 / 4;
                } else if (cnt == 1) {
                    // Look the facet up in the boundary list.
                    const FacetRec &r = fi.rec[k];
                    int64_t lo = bi.ptr[a], hi = bi.ptr[a + 1];
                    auto it = std::lower_bound(bi.rec.begin() + lo, bi.rec.begin() + hi, r,
                                               [](const FacetRec &x, const FacetRec &y) {
                                                   return x.b != y.b ? x.b < y.b : x.c < y.c;
                                               });
                    if (it == bi.rec.begin() + hi || it->b != r.b || it->c != r.c)
                        return fail(PG_ERR_MESH, "boundary facet (" + std::to_string(a) + "," + std::to_string(r.b) + "," +
                                                     std::to_string(r.c) + ") of cell " + std::to_string(r.slot / 4) + " has no tag");
                    int32_t tag = d->bfacet_tags[it->slot];
                    max_tag = std::max(max_tag, tag);
                    h.nbr[r.slot] = -int64_t(tag);
                } else {
                    return fail(PG_ERR_MESH, "a facet is shared by more than two cells");
                }
                k = k2;
            }
        }
        h.n_objects = max_tag - 1;
    }

    // Per-cell geometry.
    h.bary.assign(12 * nc, 0.0);
    h.planes.assign(16 * nc, 0.0);
    h.volume.assign(nc, 0.0);
    std::vector<int> bad(1, 0);
    parallel_for(nc, [&](int64_t b0, int64_t e0) {
        for (int64_t c = b0; c < e0; ++c) {
            double p[12];
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 3; ++j) p[3 * i + j] = h.coords[3 * h.cell_vertices[4 * c + i] + j];
            barycentric_rows(p, &h.bary[12 * c]);
            h.volume[c] = tet_volume(p);
            if (!(h.volume[c] > 0.0)) bad[0] = 1;
            for (int f = 0; f < 4; ++f) {
                double n[3], m[3];
                facet_normal(p, f, n);
                facet_midpoint(p, f, m);
                double dot = 0;
                for (int j = 0; j < 3; ++j) dot += m[j] * n[j];
                double *pl = &h.planes[16 * c + 4 * f];
                pl[0] = -dot; pl[1] = n[0]; pl[2] = n[1]; pl[3] = n[2];
            }
        }
    });
    if (bad[0]) return fail(PG_ERR_MESH, "degenerate (zero-volume) cell");

    // dv_inv: (d+1) / sum of the volumes of the cells around each dof, the
    // cells visited per vertex in ascending vertex then cell order.
    {
        std::vector<int64_t> vptr(nv + 1, 0);
        for (int64_t k = 0; k < 4 * nc; ++k) vptr[h.cell_vertices[k] + 1]++;
        for (int64_t v = 0; v < nv; ++v) vptr[v + 1] += vptr[v];
        std::vector<int64_t> vcells(4 * nc), cur(vptr.begin(), vptr.end() - 1);
        for (int64_t c = 0; c < nc; ++c)
            for (int i = 0; i < 4; ++i) vcells[cur[h.cell_vertices[4 * c + i]]++] = c;
        std::vector<double> vol(h.ndof, 0.0);
        for (int64_t v = 0; v < nv; ++v) {
            int64_t dof = d->vertex_to_dof ? d->vertex_to_dof[v] : v;
            for (int64_t k = vptr[v]; k < vptr[v + 1]; ++k) vol[dof] += h.volume[vcells[k]];
        }
        h.dv_inv.resize(h.ndof);
        for (int64_t i = 0; i < h.ndof; ++i) {
            if (!(vol[i] > 0)) return fail(PG_ERR_MESH, "a dof touches no cell");
            h.dv_inv[i] = (3 + 1.0) / vol[i];
        }
    }

    // CSR pattern over dofs, columns ascending.
    {
        const int64_t nd = h.ndof;
        std::vector<int64_t> cnt(nd + 1, 0);
        for (int64_t c = 0; c < nc; ++c)
            for (int i = 0; i < 4; ++i) cnt[h.cell_dofs[4 * c + i] + 1] += 4;
        for (int64_t i = 0; i < nd; ++i) cnt[i + 1] += cnt[i];
        std::vector<int64_t> tmp(cnt[nd]), cur(cnt.begin(), cnt.end() - 1);
        for (int64_t c = 0; c < nc; ++c)
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) tmp[cur[h.cell_dofs[4 * c + i]]++] = h.cell_dofs[4 * c + j];
        h.rowptr.assign(nd + 1, 0);
        std::vector<int64_t> rowlen(nd, 0);
        parallel_for(nd, [&](int64_t b0, int64_t e0) {
            for (int64_t r = b0; r < e0; ++r) {
                auto s = tmp.begin() + cnt[r], e = tmp.begin() + cnt[r + 1];
                std::sort(s, e);
                rowlen[r] = std::unique(s, e) - s;
            }
        });
        for (int64_t r = 0; r < nd; ++r) h.rowptr[r + 1] = h.rowptr[r] + rowlen[r];
        h.col.resize(h.rowptr[nd]);
        for (int64_t r = 0; r < nd; ++r)
            std::copy(tmp.begin() + cnt[r], tmp.begin() + cnt[r] + rowlen[r], h.col.begin() + h.rowptr[r]);
        h.K.assign(h.col.size(), 0.0);
        h.M.assign(h.col.size(), 0.0);
        // Element matrices: K_T = eps0 vol grad(l_i).grad(l_j), M_T = vol/20 (1 + delta_ij).
        for (int64_t c = 0; c < nc; ++c) {
            const double *A = &h.bary[12 * c];
            double g[4][3];
            for (int k = 0; k < 3; ++k)
                for (int j = 0; j < 3; ++j) g[k][j] = A[4 * k + 1 + j];
            for (int j = 0; j < 3; ++j) g[3][j] = -(g[0][j] + g[1][j] + g[2][j]);
            const double vol = h.volume[c];
            for (int i = 0; i < 4; ++i) {
                const int64_t r = h.cell_dofs[4 * c + i];
                for (int j = 0; j < 4; ++j) {
                    const int64_t cc = h.cell_dofs[4 * c + j];
                    auto it = std::lower_bound(h.col.begin() + h.rowptr[r], h.col.begin() + h.rowptr[r + 1], cc);
                    const int64_t k = it - h.col.begin();
                    const double gg = g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2];
                    h.K[k] += eps0 * vol * gg;
                    h.M[k] += vol / 20.0 * (i == j ? 2.0 : 1.0);
                }
            }
        }
    }

    // Boundary facet lists and Dirichlet dof kinds.
    h.bc_kind.assign(h.ndof, -1);
    h.ext_facets.clear();
    h.obj_facets.clear();
    for (int64_t c = 0; c < nc; ++c) {
        for (int f = 0; f < 4; ++f) {
            const int64_t t = h.nbr[4 * c + f];
            if (t >= 0) continue;
            const int64_t tag = -t;
            double p[12];
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 3; ++j) p[3 * i + j] = h.coords[3 * h.cell_vertices[4 * c + i] + j];
            double n[3];
            facet_normal(p, f, n);
            const double area = facet_area(p, f);
            if (tag == 1) {
                double rec[14];
                rec[0] = area;
                int k = 0;
                for (int i = 0; i < 4; ++i) {
                    if (i == f) continue;
                    for (int j = 0; j < 3; ++j) rec[1 + 3 * k + j] = p[3 * i + j];
                    ++k;
                }
                for (int j = 0; j < 3; ++j) rec[10 + j] = -1 * n[j];
                rec[13] = double(c);
                h.ext_facets.insert(h.ext_facets.end(), rec, rec + 14);
            } else {
                double rec[7] = {double(c), double(tag - 2), area, n[0], n[1], n[2], double(f)};
                h.obj_facets.insert(h.obj_facets.end(), rec, rec + 7);
            }
        }
    }
    // Exterior first, objects override (the order BCs are applied in
    // PoissonSolver::solve, punc/src/poisson.cpp:350-357).
    for (int pass = 0; pass < 2; ++pass) {
        for (int64_t c = 0; c < nc; ++c)
            for (int f = 0; f < 4; ++f) {
                const int64_t t = h.nbr[4 * c + f];
                if (t >= 0) continue;
                const int64_t tag = -t;
                if ((pass == 0) != (tag == 1)) continue;
                for (int i = 0; i < 4; ++i)
                    if (i != f) h.bc_kind[h.cell_dofs[4 * c + i]] = (tag == 1) ? 0 : tag - 1;
            }
    }

    // Bounding box and bin grid for point location.
    for (int j = 0; j < 3; ++j) { h.bbox_lo[j] = h.coords[j]; h.bbox_hi[j] = h.coords[j]; }
    for (int64_t v = 0; v < nv; ++v)
        for (int j = 0; j < 3; ++j) {
            h.bbox_lo[j] = std::min(h.bbox_lo[j], h.coords[3 * v + j]);
            h.bbox_hi[j] = std::max(h.bbox_hi[j], h.coords[3 * v + j]);
        }
    {
        double ext[3], total = 1.0;
        for (int j = 0; j < 3; ++j) { ext[j] = std::max(h.bbox_hi[j] - h.bbox_lo[j], 1e-300); total *= ext[j]; }
        const double target = std::max<double>(1.0, double(nc) / 6.0);
        const double hb = std::cbrt(total / target);
        for (int j = 0; j < 3; ++j) {
            h.nbin[j] = int32_t(std::min<double>(std::max(1.0, std::floor(ext[j] / hb)), 2048.0));
            h.bin_h[j] = ext[j] / h.nbin[j];
        }
        const int64_t nbins = int64_t(h.nbin[0]) * h.nbin[1] * h.nbin[2];
        std::vector<int64_t> cnt(nbins + 1, 0);
        auto bin_range = [&](int64_t c, int32_t lo[3], int32_t hi[3]) {
            for (int j = 0; j < 3; ++j) {
                double mn = 1e300, mx = -1e300;
                for (int i = 0; i < 4; ++i) {
                    double x = h.coords[3 * h.cell_vertices[4 * c + i] + j];
                    mn = std::min(mn, x); mx = std::max(mx, x);
                }
                lo[j] = std::max(0, std::min(h.nbin[j] - 1, int32_t(std::floor((mn - h.bbox_lo[j]) / h.bin_h[j]))));
                hi[j] = std::max(0, std::min(h.nbin[j] - 1, int32_t(std::floor((mx - h.bbox_lo[j]) / h.bin_h[j]))));
            }
        };
        for (int pass = 0; pass < 2; ++pass) {
            std::vector<int64_t> cur;
            if (pass == 1) {
                for (int64_t b = 0; b < nbins; ++b) cnt[b + 1] += cnt[b];
                h.bin_ptr = cnt;
                h.bin_cells.assign(cnt[nbins], 0);
                cur.assign(cnt.begin(), cnt.end() - 1);
            }
            for (int64_t c = 0; c < nc; ++c) {
                int32_t lo[3], hi[3];
                bin_range(c, lo, hi);
                for (int32_t a = lo[0]; a <= hi[0]; ++a)
                    for (int32_t b = lo[1]; b <= hi[1]; ++b)
                        for (int32_t e = lo[2]; e <= hi[2]; ++e) {
                            int64_t bin = (int64_t(a) * h.nbin[1] + b) * h.nbin[2] + e;
                            if (pass == 0) cnt[bin + 1]++;
                            else h.bin_cells[cur[bin]++] = int32_t(c);
                        }
            }
        }
    }
    return PG_OK;
}

}  // namespace pg

extern "C" {

const char *pg_last_error(void) { return pg::last_error_cstr(); }
int32_t pg_abi_version(void) { return PG_ABI_VERSION; }

int pg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    if (!ctr || !key || !out) return pg::fail(PG_ERR_ARG, "pg_philox4x32_10: NULL argument");
    const pg::Philox4 r = pg::philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.v[i];
    return PG_OK;
}

int pg_mesh_build(const pg_mesh_desc *desc, double eps0, pg_mesh **out) {
    if (!out) return pg::fail(PG_ERR_ARG, "pg_mesh_build: out is NULL");
    *out = nullptr;
    pg_mesh *m = new (std::nothrow) pg_mesh;
    if (!m) return pg::fail(PG_ERR_ARG, "pg_mesh_build: out of host memory");
    int rc;
    try {
        rc = pg::build_mesh(desc, eps0, m->h);
    } catch (const std::exception &e) {
        rc = pg::fail(PG_ERR_ARG, std::string("pg_mesh_build: ") + e.what());
    }
    if (rc != PG_OK) { delete m; return rc; }
    *out = m;
    return PG_OK;
}

int pg_mesh_array(const pg_mesh *mesh, int32_t which, const void **data, int64_t *count) {
    if (!mesh || !data || !count) return pg::fail(PG_ERR_ARG, "pg_mesh_array: NULL argument");
    const pg::HostMesh &h = mesh->h;
    switch (which) {
    case PG_T_CELL_VERTICES: *data = h.cell_vertices.data(); *count = (int64_t)h.cell_vertices.size(); break;
    case PG_T_BARYCENTRIC: *data = h.bary.data(); *count = (int64_t)h.bary.size(); break;
    case PG_T_PLANES: *data = h.planes.data(); *count = (int64_t)h.planes.size(); break;
    case PG_T_NEIGHBOURS: *data = h.nbr.data(); *count = (int64_t)h.nbr.size(); break;
    case PG_T_CELL_DOFS: *data = h.cell_dofs.data(); *count = (int64_t)h.cell_dofs.size(); break;
    case PG_T_VOLUME: *data = h.volume.data(); *count = (int64_t)h.volume.size(); break;
    case PG_T_DV_INV: *data = h.dv_inv.data(); *count = (int64_t)h.dv_inv.size(); break;
    case PG_T_CSR_ROWPTR: *data = h.rowptr.data(); *count = (int64_t)h.rowptr.size(); break;
    case PG_T_CSR_COL: *data = h.col.data(); *count = (int64_t)h.col.size(); break;
    case PG_T_STIFFNESS: *data = h.K.data(); *count = (int64_t)h.K.size(); break;
    case PG_T_MASS: *data = h.M.data(); *count = (int64_t)h.M.size(); break;
    case PG_T_EXT_FACETS: *data = h.ext_facets.data(); *count = (int64_t)h.ext_facets.size(); break;
    case PG_T_BC_KIND: *data = h.bc_kind.data(); *count = (int64_t)h.bc_kind.size(); break;
    case PG_T_OBJ_FACETS: *data = h.obj_facets.data(); *count = (int64_t)h.obj_facets.size(); break;
    default: return pg::fail(PG_ERR_ARG, "pg_mesh_array: unknown table");
    }
    return PG_OK;
}

int pg_mesh_free(pg_mesh *mesh) {
    delete mesh;
    return PG_OK;
}

}  // extern "C"
