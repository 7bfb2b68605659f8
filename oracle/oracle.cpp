// ORACLE - test infrastructure only.  A CPU restatement of the PUNC++
// per-timestep particle path, used by tests/, the smoke check and bench.py's
// CPU-baseline leg to check and time the GPU engine.  Never part of the
// product path.
//
// It keeps the reference's data model: AoS particles {x, v, q, m} bucketed in
// per-cell std::vectors, cells visited in id order, particles in vector
// order, Population::update's push_back / swap-with-back bookkeeping.  Each
// function cites the reference file:line it restates (paths relative to the
// PUNC++ tree).
//
// Parity status: the reference cannot be built here (DOLFIN 2019.1, FFC,
// PETSc and Boost are absent) and ships no golden vectors, so parity with the
// reference binary is UNPINNED.  The arithmetic of DOLFIN's
// TetrahedronCell::normal and MeshEntity::midpoint is restated from the
// published DOLFIN 2019.1.0 source; the cell volume, facet area, P1 element
// matrices (FFC for punc/ufl/Potential3D.ufl) and the DG0 gradient are
// restated from the mathematics.  The analytic known answers of the
// reference's demos (capacitance, Langmuir frequency, orbit, flux count) are
// checked against this oracle in tests/test_oracle_known_answers.py.
//
// Compile with -ffp-contract=off and without -march (the reference's Release
// build, punc/CMakeLists.txt).
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

namespace {

struct Particle {            // punc/include/punc/population.h:74-94 (+ a test id)
    double x[3];
    double v[3];
    double q;
    double m;
    int64_t id;
};

struct Cell {                // punc/include/punc/population.h:179-231
    int64_t id;
    int64_t vertices[4];     // ascending global index (DOLFIN ordered mesh)
    std::array<double, 12> vertex_coordinates;
    double barycentric_matrix[12];
    std::vector<long> facet_adjacents;
    std::vector<double> facet_plane_coeffs;
    std::vector<Particle> particles;
    int64_t dofs[4];
    double volume;

    // Cell<3>::init_barycentric_matrix (punc/src/population.cpp:181-240)
    void init_barycentric_matrix() {
        double x1 = vertex_coordinates[0], y1 = vertex_coordinates[1], z1 = vertex_coordinates[2];
        double x2 = vertex_coordinates[3], y2 = vertex_coordinates[4], z2 = vertex_coordinates[5];
        double x3 = vertex_coordinates[6], y3 = vertex_coordinates[7], z3 = vertex_coordinates[8];
        double x4 = vertex_coordinates[9], y4 = vertex_coordinates[10], z4 = vertex_coordinates[11];
        double x13 = x1 - x3; double y13 = y1 - y3; double z13 = z1 - z3;
        double x14 = x1 - x4; double y14 = y1 - y4; double z14 = z1 - z4;
        double x24 = x2 - x4; double y24 = y2 - y4; double z24 = z2 - z4;
        double x31 = x3 - x1; double y31 = y3 - y1; double z31 = z3 - z1;
        double x32 = x3 - x2; double y32 = y3 - y2; double z32 = z3 - z2;
        double x34 = x3 - x4; double y34 = y3 - y4; double z34 = z3 - z4;
        double x42 = x4 - x2; double y42 = y4 - y2; double z42 = z4 - z2;
        double x43 = x4 - x3; double y43 = y4 - y3; double z43 = z4 - z3;
        double V01 = (x2 * (y3 * z4 - y4 * z3) + x3 * (y4 * z2 - y2 * z4) + x4 * (y2 * z3 - y3 * z2)) / 6.0;
        double V02 = (x1 * (y4 * z3 - y3 * z4) + x3 * (y1 * z4 - y4 * z1) + x4 * (y3 * z1 - y1 * z3)) / 6.0;
        double V03 = (x1 * (y2 * z4 - y4 * z2) + x2 * (y4 * z1 - y1 * z4) + x4 * (y1 * z2 - y2 * z1)) / 6.0;
        double V04 = (x1 * (y3 * z2 - y2 * z3) + x2 * (y1 * z3 - y3 * z1) + x3 * (y2 * z1 - y1 * z2)) / 6.0;
        double V = V01 + V02 + V03 + V04;
        double V6 = 6 * V;
        double *A = barycentric_matrix;
        A[0] = V01 / V; A[4] = V02 / V; A[8] = V03 / V;
        A[1] = (y42 * z32 - y32 * z42) / V6;
        A[5] = (y31 * z43 - y34 * z13) / V6;
        A[9] = (y24 * z14 - y14 * z24) / V6;
        A[2] = (x32 * z42 - x42 * z32) / V6;
        A[6] = (x43 * z31 - x13 * z34) / V6;
        A[10] = (x14 * z24 - x24 * z14) / V6;
        A[3] = (x42 * y32 - x32 * y42) / V6;
        A[7] = (x31 * y43 - x34 * y13) / V6;
        A[11] = (x24 * y14 - x14 * y24) / V6;
    }

    // Cell<3>::barycentric (punc/include/punc/population.h:885-893)
    void barycentric(const double *x, double *y) const {
        const double *A = barycentric_matrix;
        y[0] = A[0] + A[1] * x[0] + A[2] * x[1] + A[3] * x[2];
        y[1] = A[4] + A[5] * x[0] + A[6] * x[1] + A[7] * x[2];
        y[2] = A[8] + A[9] * x[0] + A[10] * x[1] + A[11] * x[2];
        y[3] = 1 - y[0] - y[1] - y[2];
    }

    // DOLFIN 2019.1.0 TetrahedronCell::normal(cell, facet): cross product of
    // the facet's edge vectors from its first vertex, normalised, flipped to
    // point away from the opposite vertex.
    std::array<double, 3> normal(int facet) const {
        int f[3], k = 0;
        for (int i = 0; i < 4; ++i) if (i != facet) f[k++] = i;
        const double *P0 = &vertex_coordinates[3 * facet];
        const double *P1 = &vertex_coordinates[3 * f[0]];
        const double *P2 = &vertex_coordinates[3 * f[1]];
        const double *P3 = &vertex_coordinates[3 * f[2]];
        double V0[3], V1[3], V2[3];
        for (int j = 0; j < 3; ++j) { V0[j] = P0[j] - P1[j]; V1[j] = P2[j] - P1[j]; V2[j] = P3[j] - P1[j]; }
        double n[3] = {V1[1] * V2[2] - V1[2] * V2[1], V1[2] * V2[0] - V1[0] * V2[2], V1[0] * V2[1] - V1[1] * V2[0]};
        double norm = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int j = 0; j < 3; ++j) n[j] /= norm;
        if (n[0] * V0[0] + n[1] * V0[1] + n[2] * V0[2] > 0)
            for (int j = 0; j < 3; ++j) n[j] *= -1.0;
        return {n[0], n[1], n[2]};
    }

    // DOLFIN 2019.1.0 MeshEntity::midpoint: running vertex sum / vertex count.
    std::array<double, 3> facet_midpoint(int facet) const {
        double x = 0.0, y = 0.0, z = 0.0;
        std::size_t num_vertices = 0;
        for (int i = 0; i < 4; ++i) {
            if (i == facet) continue;
            x += vertex_coordinates[3 * i];
            y += vertex_coordinates[3 * i + 1];
            z += vertex_coordinates[3 * i + 2];
            num_vertices++;
        }
        x /= double(num_vertices); y /= double(num_vertices); z /= double(num_vertices);
        return {x, y, z};
    }
};

// Portable Philox4x32-10 (Salmon et al., SC'11) and the stream layout of the
// engine's injection: key = seed, counter = (block, facet, species, step).
struct Philox {
    static void round10(uint32_t c[4], uint32_t k0, uint32_t k1) {
        for (int r = 0; r < 10; ++r) {
            const uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
            const uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
            const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
            const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
            const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
            c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
            k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
        }
    }
};

struct Stream {
    uint32_t k0, k1, c1, c2, c3, block = 0;
    bool have = false;
    double cached = 0;
    Stream(uint64_t seed, uint32_t a, uint32_t b, uint32_t c) : k0(uint32_t(seed)), k1(uint32_t(seed >> 32)), c1(a), c2(b), c3(c) {}
    static double res53(uint32_t a, uint32_t b) {
        return (double(a >> 5) * 67108864.0 + double(b >> 6)) * (1.0 / 9007199254740992.0);
    }
    double operator()() {
        if (have) { have = false; return cached; }
        uint32_t c[4] = {block, c1, c2, c3};
        Philox::round10(c, k0, k1);
        ++block;
        cached = res53(c[2], c[3]);
        have = true;
        return res53(c[0], c[1]);
    }
};

// exp from Cody-Waite reduction by ln2 (24-bit head) and the degree-13
// Taylor polynomial, so CPU and GPU accept/reject identically.
double exp_series(double x) {
    if (x != x) return x;
    if (x > 709.5) return HUGE_VAL;
    if (x < -745.0) return 0.0;
    const double kf = std::floor(x * 0x1.71547652b82fep+0 + 0.5);
    const double r = (x - kf * 0x1.62e4300000000p-1) - kf * -0x1.05c610ca86c39p-29;
    static const double c[14] = {0x1.6124613a86d09p-33, 0x1.1eed8eff8d898p-29, 0x1.ae64567f544e4p-26,
                                 0x1.27e4fb7789f5cp-22, 0x1.71de3a556c734p-19, 0x1.a01a01a01a01ap-16,
                                 0x1.a01a01a01a01ap-13, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7,
                                 0x1.5555555555555p-5, 0x1.5555555555555p-3, 0.5, 1.0, 1.0};
    double p = c[0];
    for (int i = 1; i < 14; ++i) p = p * r + c[i];
    int k = int(kf);
    double extra = 1.0;
    if (k < -1020) { k += 1000; extra = 0x1p-1000; }
    const uint64_t bits = uint64_t(int64_t(k) + 1023) << 52;
    double two_k;
    std::memcpy(&two_k, &bits, 8);
    return (p * two_k) * extra;
}

struct ExtFacet {            // punc/include/punc/mesh.h:38-44
    double area;
    double vertices[9];
    double normal[3];        // inward
    int64_t cell;
};

struct SpeciesFlux {         // Maxwellian part of punc/include/punc/distributions.h:52-249
    double q, m, n, vth, vd[3], vdf_range;
    double vth2, factor;
    double domain[6];
    std::vector<double> num_particles, pdf_max;
};

struct Oracle {
    int64_t nv = 0, nc = 0, ndof = 0;
    std::vector<double> coords;
    std::vector<int64_t> v2d;
    std::vector<Cell> cells;
    std::vector<double> dv_inv;
    std::vector<int64_t> rowptr, col;
    std::vector<double> K, M;
    std::vector<ExtFacet> ext;
    std::vector<double> ofac;   // cell, object, area, n(3), facet
    std::vector<int64_t> bc_kind;
    double eps0 = 1.0;
    // locate acceleration: uniform grid of cell lists
    double glo[3], gh[3];
    int gn[3];
    std::vector<std::vector<int64_t>> grid;
    std::vector<SpeciesFlux> flux;
    int64_t next_id = 0;
};

// ---- setup -------------------------------------------------------------------

int build(Oracle &o, const double *coords, int64_t nv, const int64_t *cells, int64_t nc, const int64_t *bfv,
          const int32_t *btag, int64_t nb, const int64_t *v2d, int64_t ndof, double eps0) {
    o.nv = nv; o.nc = nc; o.eps0 = eps0;
    o.coords.assign(coords, coords + 3 * nv);
    o.ndof = v2d ? ndof : nv;
    o.v2d.resize(nv);
    for (int64_t v = 0; v < nv; ++v) o.v2d[v] = v2d ? v2d[v] : v;
    std::map<std::array<int64_t, 3>, int32_t> tags;
    for (int64_t k = 0; k < nb; ++k) {
        std::array<int64_t, 3> t = {bfv[3 * k], bfv[3 * k + 1], bfv[3 * k + 2]};
        std::sort(t.begin(), t.end());
        tags[t] = btag[k];
    }
    o.cells.resize(nc);
    // facets sorted by vertex triple to find neighbours
    std::vector<std::pair<std::array<int64_t, 3>, int64_t>> fl(4 * nc);
    for (int64_t c = 0; c < nc; ++c) {
        Cell &cell = o.cells[c];
        cell.id = c;
        int64_t v[4] = {cells[4 * c], cells[4 * c + 1], cells[4 * c + 2], cells[4 * c + 3]};
        std::sort(v, v + 4);
        for (int i = 0; i < 4; ++i) {
            cell.vertices[i] = v[i];
            cell.dofs[i] = o.v2d[v[i]];
            for (int j = 0; j < 3; ++j) cell.vertex_coordinates[3 * i + j] = coords[3 * v[i] + j];
        }
        cell.init_barycentric_matrix();
        for (int f = 0; f < 4; ++f) {
            std::array<int64_t, 3> t;
            int k = 0;
            for (int i = 0; i < 4; ++i) if (i != f) t[k++] = v[i];
            fl[4 * c + f] = {t, 4 * c + f};
        }
    }
    std::sort(fl.begin(), fl.end());
    std::vector<long> adj(4 * nc, 0);
    for (size_t k = 0; k < fl.size();) {
        size_t e = k + 1;
        while (e < fl.size() && fl[e].first == fl[k].first) ++e;
        if (e - k == 2) {
            adj[fl[k].second] = fl[k + 1].second / 4;
            adj[fl[k + 1].second] = fl[k].second / 4;
        } else if (e - k == 1) {
            auto it = tags.find(fl[k].first);
            if (it == tags.end()) return 3;
            adj[fl[k].second] = -1 * (long)it->second;
        } else {
            return 3;
        }
        k = e;
    }
    // Population::init_localizer (punc/include/punc/population.h:345-389)
    for (auto &cell : o.cells) {
        cell.facet_adjacents.clear();
        cell.facet_plane_coeffs.clear();
        for (int i = 0; i < 4; ++i) {
            cell.facet_adjacents.push_back(adj[4 * cell.id + i]);
            double dot_product = 0;
            for (int j = 0; j < 3; ++j) dot_product += cell.facet_midpoint(i)[j] * cell.normal(i)[j];
            cell.facet_plane_coeffs.push_back(-dot_product);
            for (int j = 0; j < 3; ++j) cell.facet_plane_coeffs.push_back(cell.normal(i)[j]);
        }
        const double *p = cell.vertex_coordinates.data();
        double a[3], b[3], d[3];
        for (int j = 0; j < 3; ++j) { a[j] = p[3 + j] - p[j]; b[j] = p[6 + j] - p[j]; d[j] = p[9 + j] - p[j]; }
        const double det = a[0] * (b[1] * d[2] - b[2] * d[1]) - a[1] * (b[0] * d[2] - b[2] * d[0]) + a[2] * (b[0] * d[1] - b[1] * d[0]);
        cell.volume = std::fabs(det) / 6.0;
    }
    // element_volume (punc/src/distributor.cpp:35-69): per vertex in order, the
    // volumes of its cells in ascending cell order, into the vertex's dof.
    {
        std::vector<std::vector<int64_t>> vc(nv);
        for (int64_t c = 0; c < nc; ++c)
            for (int i = 0; i < 4; ++i) vc[o.cells[c].vertices[i]].push_back(c);
        std::vector<double> volumes(o.ndof, 0.0);
        for (int64_t v = 0; v < nv; ++v)
            for (int64_t c : vc[v]) volumes[o.v2d[v]] += o.cells[c].volume;
        o.dv_inv.resize(o.ndof);
        for (int64_t i = 0; i < o.ndof; ++i) o.dv_inv[i] = (3 + 1.0) / volumes[i];
    }
    // P1 stiffness eps0*grad.grad and consistent mass (punc/ufl/Potential3D.ufl)
    {
        struct Entry { int64_t col; double k, m; };
        std::vector<std::vector<Entry>> rows(o.ndof);
        for (auto &cell : o.cells) {
            const double *A = cell.barycentric_matrix;
            double g[4][3];
            for (int k = 0; k < 3; ++k) for (int j = 0; j < 3; ++j) g[k][j] = A[4 * k + 1 + j];
            for (int j = 0; j < 3; ++j) g[3][j] = -(g[0][j] + g[1][j] + g[2][j]);
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) {
                    auto &row = rows[cell.dofs[i]];
                    Entry *e = nullptr;
                    for (auto &x : row) if (x.col == cell.dofs[j]) { e = &x; break; }
                    if (!e) { row.push_back(Entry{cell.dofs[j], 0.0, 0.0}); e = &row.back(); }
                    const double gg = g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2];
                    e->k += eps0 * cell.volume * gg;
                    e->m += cell.volume / 20.0 * (i == j ? 2.0 : 1.0);
                }
        }
        o.rowptr.assign(o.ndof + 1, 0);
        for (int64_t r = 0; r < o.ndof; ++r) {
            std::sort(rows[r].begin(), rows[r].end(), [](const Entry &a, const Entry &b) { return a.col < b.col; });
            for (auto &e : rows[r]) { o.col.push_back(e.col); o.K.push_back(e.k); o.M.push_back(e.m); }
            o.rowptr[r + 1] = (int64_t)o.col.size();
        }
    }
    // Mesh::exterior_boundaries (punc/src/mesh.cpp:166-236) and object facets
    o.bc_kind.assign(o.ndof, -1);
    for (auto &cell : o.cells)
        for (int f = 0; f < 4; ++f) {
            const long t = cell.facet_adjacents[f];
            if (t >= 0) continue;
            const double *p = cell.vertex_coordinates.data();
            int q[3], k = 0;
            for (int i = 0; i < 4; ++i) if (i != f) q[k++] = i;
            double b[3], d[3];
            for (int j = 0; j < 3; ++j) { b[j] = p[3 * q[1] + j] - p[3 * q[0] + j]; d[j] = p[3 * q[2] + j] - p[3 * q[0] + j]; }
            const double cx = b[1] * d[2] - b[2] * d[1], cy = b[2] * d[0] - b[0] * d[2], cz = b[0] * d[1] - b[1] * d[0];
            const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
            const auto n = cell.normal(f);
            if (t == -1) {
                ExtFacet e;
                e.area = area;
                for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) e.vertices[3 * i + j] = p[3 * q[i] + j];
                for (int j = 0; j < 3; ++j) e.normal[j] = -1 * n[j];
                e.cell = cell.id;
                o.ext.push_back(e);
            } else {
                const double rec[7] = {double(cell.id), double(-t - 2), area, n[0], n[1], n[2], double(f)};
                o.ofac.insert(o.ofac.end(), rec, rec + 7);
            }
        }
    for (int pass = 0; pass < 2; ++pass)
        for (auto &cell : o.cells)
            for (int f = 0; f < 4; ++f) {
                const long t = cell.facet_adjacents[f];
                if (t >= 0 || (pass == 0) != (t == -1)) continue;
                for (int i = 0; i < 4; ++i) if (i != f) o.bc_kind[cell.dofs[i]] = (t == -1) ? 0 : -t - 1;
            }
    // locate grid
    for (int j = 0; j < 3; ++j) { o.glo[j] = 1e300; double hi = -1e300; for (int64_t v = 0; v < nv; ++v) { o.glo[j] = std::min(o.glo[j], coords[3 * v + j]); hi = std::max(hi, coords[3 * v + j]); } o.gn[j] = std::max<int>(1, (int)std::cbrt((double)nc / 6.0)); o.gh[j] = std::max(hi - o.glo[j], 1e-300) / o.gn[j]; }
    o.grid.assign((size_t)o.gn[0] * o.gn[1] * o.gn[2], {});
    for (auto &cell : o.cells) {
        int lo[3], hi[3];
        for (int j = 0; j < 3; ++j) {
            double mn = 1e300, mx = -1e300;
            for (int i = 0; i < 4; ++i) { mn = std::min(mn, cell.vertex_coordinates[3 * i + j]); mx = std::max(mx, cell.vertex_coordinates[3 * i + j]); }
            lo[j] = std::max(0, std::min(o.gn[j] - 1, (int)std::floor((mn - o.glo[j]) / o.gh[j])));
            hi[j] = std::max(0, std::min(o.gn[j] - 1, (int)std::floor((mx - o.glo[j]) / o.gh[j])));
        }
        for (int a = lo[0]; a <= hi[0]; ++a) for (int b = lo[1]; b <= hi[1]; ++b) for (int e = lo[2]; e <= hi[2]; ++e)
            o.grid[((size_t)a * o.gn[1] + b) * o.gn[2] + e].push_back(cell.id);
    }
    return 0;
}

// The lowest-index cell whose four plane values are all <= 0, or -1.
// (Stands in for the BoundingBoxTree query of locate, punc/src/population.cpp:24-39;
// the two agree for every point strictly inside a cell.)
long locate(const Oracle &o, const double *x) {
    int b[3];
    for (int j = 0; j < 3; ++j) {
        const double f = std::floor((x[j] - o.glo[j]) / o.gh[j]);
        if (!(f >= -1.0 && f <= (double)o.gn[j])) return -1;
        b[j] = f < 0 ? 0 : (f >= o.gn[j] ? o.gn[j] - 1 : (int)f);
    }
    const auto &lst = o.grid[((size_t)b[0] * o.gn[1] + b[1]) * o.gn[2] + b[2]];
    long best = -1;
    for (int64_t c : lst) {
        const double *co = o.cells[c].facet_plane_coeffs.data();
        bool in = true;
        for (int i = 0; i < 4 && in; ++i) {
            double proj = co[4 * i];
            for (int j = 0; j < 3; ++j) proj += co[4 * i + 1 + j] * x[j];
            if (proj > 0) in = false;
        }
        if (in && (best < 0 || c < best)) best = (long)c;
    }
    return best;
}

// Population::relocate_fast (punc/include/punc/population.h:539-569).  The
// tail recursion is a loop here, with a step limit (LONG_MIN when reached).
long relocate_fast(const Oracle &o, const double *p, long cell_id) {
    for (int depth = 0; depth <= 100000; ++depth) {
        const double *coeffs = o.cells[cell_id].facet_plane_coeffs.data();
        long next = cell_id;
        for (int i = 0; i < 4; ++i) {
            double proj = *coeffs++;
            for (int j = 0; j < 3; j++) proj += *coeffs++ * p[j];
            if (proj > 0) { next = o.cells[cell_id].facet_adjacents[i]; break; }
        }
        if (next == cell_id || next < 0) return next;
        cell_id = next;
    }
    return LONG_MIN;
}

// Range split for the threaded variants (cells are the unit of work).
template <class F>
void for_cells(int64_t nc, int nthreads, F f) {
    if (nthreads <= 1) { f(0, nc, 0); return; }
    std::vector<std::thread> ts;
    const int64_t chunk = (nc + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        const int64_t b = t * chunk, e = std::min(nc, b + chunk);
        if (b >= e) break;
        ts.emplace_back([=] { f(b, e, t); });
    }
    for (auto &t : ts) t.join();
}

}  // namespace

extern "C" {

void *or_create(const double *coords, int64_t nv, const int64_t *cells, int64_t nc, const int64_t *bfv,
                const int32_t *btag, int64_t nb, const int64_t *v2d, int64_t ndof, double eps0, int32_t *status) {
    Oracle *o = new Oracle;
    const int rc = build(*o, coords, nv, cells, nc, bfv, btag, nb, v2d, ndof, eps0);
    if (status) *status = rc;
    if (rc) { delete o; return nullptr; }
    return o;
}

void or_free(void *h) { delete static_cast<Oracle *>(h); }

// Table sizes: 0 bary(12) 1 planes(16) 2 nbr(4) 3 dofs(4) 4 volume 5 dv_inv
// 6 rowptr 7 col 8 K 9 M 10 ext facets(14) 11 bc_kind 12 obj facets(7) 13 cell vertices(4)
int64_t or_table_size(void *h, int32_t which) {
    const Oracle &o = *static_cast<Oracle *>(h);
    switch (which) {
    case 0: return 12 * o.nc;
    case 1: return 16 * o.nc;
    case 2: case 3: case 13: return 4 * o.nc;
    case 4: return o.nc;
    case 5: return o.ndof;
    case 6: return o.ndof + 1;
    case 7: case 8: case 9: return (int64_t)o.col.size();
    case 10: return 14 * (int64_t)o.ext.size();
    case 11: return o.ndof;
    case 12: return (int64_t)o.ofac.size();
    }
    return -1;
}

void or_table(void *h, int32_t which, void *out) {
    const Oracle &o = *static_cast<Oracle *>(h);
    double *d = static_cast<double *>(out);
    int64_t *l = static_cast<int64_t *>(out);
    for (int64_t c = 0; c < o.nc && which <= 4; ++c) {
        const Cell &cell = o.cells[c];
        if (which == 0) for (int k = 0; k < 12; ++k) d[12 * c + k] = cell.barycentric_matrix[k];
        if (which == 1) for (int k = 0; k < 16; ++k) d[16 * c + k] = cell.facet_plane_coeffs[k];
        if (which == 2) for (int k = 0; k < 4; ++k) l[4 * c + k] = cell.facet_adjacents[k];
        if (which == 3) for (int k = 0; k < 4; ++k) l[4 * c + k] = cell.dofs[k];
        if (which == 4) d[c] = cell.volume;
    }
    if (which == 13) for (int64_t c = 0; c < o.nc; ++c) for (int k = 0; k < 4; ++k) l[4 * c + k] = o.cells[c].vertices[k];
    if (which == 5) std::copy(o.dv_inv.begin(), o.dv_inv.end(), d);
    if (which == 6) std::copy(o.rowptr.begin(), o.rowptr.end(), l);
    if (which == 7) std::copy(o.col.begin(), o.col.end(), l);
    if (which == 8) std::copy(o.K.begin(), o.K.end(), d);
    if (which == 9) std::copy(o.M.begin(), o.M.end(), d);
    if (which == 10)
        for (size_t f = 0; f < o.ext.size(); ++f) {
            const ExtFacet &e = o.ext[f];
            d[14 * f] = e.area;
            for (int k = 0; k < 9; ++k) d[14 * f + 1 + k] = e.vertices[k];
            for (int k = 0; k < 3; ++k) d[14 * f + 10 + k] = e.normal[k];
            d[14 * f + 13] = (double)e.cell;
        }
    if (which == 11) std::copy(o.bc_kind.begin(), o.bc_kind.end(), l);
    if (which == 12) std::copy(o.ofac.begin(), o.ofac.end(), d);
}

void or_locate(void *h, const double *xs, int64_t n, int64_t *out) {
    const Oracle &o = *static_cast<Oracle *>(h);
    for (int64_t i = 0; i < n; ++i) out[i] = locate(o, xs + 3 * i);
}

// Population::add_particles(xs, vs, q, m) (punc/include/punc/population.h:411-435);
// points outside the mesh are dropped.  Ids continue a running counter.
int64_t or_add_particles(void *h, const double *xs, const double *vs, int64_t n, double q, double m) {
    Oracle &o = *static_cast<Oracle *>(h);
    int64_t added = 0;
    for (int64_t i = 0; i < n; ++i) {
        const long c = locate(o, xs + 3 * i);
        if (c >= 0) {
            Particle p;
            for (int j = 0; j < 3; ++j) { p.x[j] = xs[3 * i + j]; p.v[j] = vs[3 * i + j]; }
            p.q = q; p.m = m; p.id = o.next_id + i;
            o.cells[c].particles.push_back(p);
            ++added;
        }
    }
    o.next_id += n;
    return added;
}

int64_t or_num_particles(void *h) {
    const Oracle &o = *static_cast<Oracle *>(h);
    int64_t n = 0;
    for (auto &c : o.cells) n += (int64_t)c.particles.size();
    return n;
}

// Particles in storage order (cell by cell, vector order).
void or_get_particles(void *h, double *x, double *v, double *q, double *m, int64_t *cell, int64_t *id) {
    const Oracle &o = *static_cast<Oracle *>(h);
    int64_t k = 0;
    for (auto &c : o.cells)
        for (auto &p : c.particles) {
            for (int j = 0; j < 3; ++j) { x[3 * k + j] = p.x[j]; v[3 * k + j] = p.v[j]; }
            q[k] = p.q; m[k] = p.m; cell[k] = c.id; id[k] = p.id;
            ++k;
        }
}

// Replace all particles (cell given), used to resynchronise with the engine.
void or_set_particles(void *h, const double *x, const double *v, const double *q, const double *m,
                      const int64_t *cell, const int64_t *id, int64_t n) {
    Oracle &o = *static_cast<Oracle *>(h);
    for (auto &c : o.cells) c.particles.clear();
    for (int64_t k = 0; k < n; ++k) {
        Particle p;
        for (int j = 0; j < 3; ++j) { p.x[j] = x[3 * k + j]; p.v[j] = v[3 * k + j]; }
        p.q = q[k]; p.m = m[k]; p.id = id[k];
        o.cells[cell[k]].particles.push_back(p);
        o.next_id = std::max(o.next_id, id[k] + 1);
    }
}

// EFieldDG0 (punc/src/efield.cpp:95-99, punc/ufl/EFieldDG03D.ufl): per cell
// E = -((phi0-phi3) g0 + (phi1-phi3) g1 + (phi2-phi3) g2) + E0.
void or_efield_dg0(void *h, const double *phi, const double *E0, double *E) {
    const Oracle &o = *static_cast<Oracle *>(h);
    for (const Cell &c : o.cells) {
        const double *A = c.barycentric_matrix;
        const double p3 = phi[c.dofs[3]];
        const double a = phi[c.dofs[0]] - p3, b = phi[c.dofs[1]] - p3, e = phi[c.dofs[2]] - p3;
        for (int d = 0; d < 3; ++d) {
            const double g = a * A[1 + d] + b * A[5 + d] + e * A[9 + d];
            E[3 * c.id + d] = -g + (E0 ? E0[d] : 0.0);
        }
    }
}

// boris with a DG0 field and uniform B (punc/include/punc/pusher.h:397-510).
// The DG0 basis is the unit vectors, so the evaluated field is E[cell].
double or_boris(void *h, const double *E, const double *B, double dt, int32_t nthreads) {
    Oracle &o = *static_cast<Oracle *>(h);
    std::vector<double> part(std::max(1, nthreads), 0.0);
    for_cells(o.nc, nthreads, [&](int64_t cb, int64_t ce, int t) {
        double KE = 0.0;
        double v_minus[3], v_prime[3], v_plus[3], tt[3], s[3];
        for (int64_t cid = cb; cid < ce; ++cid) {
            Cell &cell = o.cells[cid];
            const double *Ei = E + 3 * cid;
            for (auto &particle : cell.particles) {
                const double m = particle.m, q = particle.q;
                const double *vel = particle.v;
                double t_mag2 = 0.0;
                for (int i = 0; i < 3; ++i) { tt[i] = std::tan((dt * q / (2.0 * m)) * B[i]); t_mag2 += tt[i] * tt[i]; }
                for (int i = 0; i < 3; ++i) s[i] = 2 * tt[i] / (1 + t_mag2);
                for (int i = 0; i < 3; ++i) v_minus[i] = vel[i] + 0.5 * dt * (q / m) * Ei[i];
                for (int i = 0; i < 3; i++) KE += 0.5 * m * v_minus[i] * v_minus[i];
                const double c1[3] = {v_minus[1] * tt[2] - v_minus[2] * tt[1], -v_minus[0] * tt[2] + v_minus[2] * tt[0],
                                      v_minus[0] * tt[1] - v_minus[1] * tt[0]};
                for (int i = 0; i < 3; ++i) v_prime[i] = v_minus[i] + c1[i];
                const double c2[3] = {v_prime[1] * s[2] - v_prime[2] * s[1], -v_prime[0] * s[2] + v_prime[2] * s[0],
                                      v_prime[0] * s[1] - v_prime[1] * s[0]};
                for (int i = 0; i < 3; ++i) v_plus[i] = v_minus[i] + c2[i];
                for (int i = 0; i < 3; ++i) particle.v[i] = v_plus[i] + 0.5 * dt * (q / m) * Ei[i];
            }
        }
        part[t] = KE;
    });
    double KE = 0.0;
    for (double p : part) KE += p;
    return KE;
}

// accel with a DG0 field (punc/include/punc/pusher.h:66-130).
double or_accel(void *h, const double *E, double dt, int32_t nthreads) {
    Oracle &o = *static_cast<Oracle *>(h);
    std::vector<double> part(std::max(1, nthreads), 0.0);
    for_cells(o.nc, nthreads, [&](int64_t cb, int64_t ce, int t) {
        double KE = 0.0;
        for (int64_t cid = cb; cid < ce; ++cid) {
            Cell &cell = o.cells[cid];
            for (auto &particle : cell.particles) {
                double Ei[3] = {E[3 * cid], E[3 * cid + 1], E[3 * cid + 2]};
                const double m = particle.m, q = particle.q;
                const double *vel = particle.v;
                for (int j = 0; j < 3; j++) {
                    Ei[j] *= dt * (q / m);
                    KE += 0.5 * m * vel[j] * (vel[j] + Ei[j]);
                }
                for (int j = 0; j < 3; j++) particle.v[j] += Ei[j];
            }
        }
        part[t] = KE;
    });
    double KE = 0.0;
    for (double p : part) KE += p;
    return KE;
}

// ESolver right-hand side (punc/src/efield.cpp:70-75, punc/ufl/EField3D.ufl:
// L = inner(-grad(phi), v) dx): for a P1 phi the gradient is constant on a
// cell, and the integral of lambda_i over the cell is vol/4, so
// b[d][c] = sum over the cells T of dof d of (vol_T / 4) (-grad phi_T)_c.
// The gradient uses the DG0 field's arithmetic (or_efield_dg0 with E0 = 0).
void or_esolver_rhs(void *h, const double *phi, double *b) {
    const Oracle &o = *static_cast<Oracle *>(h);
    std::vector<double> E(3 * (size_t)o.nc);
    or_efield_dg0(h, phi, nullptr, E.data());
    for (int64_t i = 0; i < 3 * o.ndof; ++i) b[i] = 0.0;
    for (const Cell &c : o.cells) {
        const double w = 0.25 * c.volume;
        for (int i = 0; i < 4; ++i)
            for (int d = 0; d < 3; ++d) b[3 * c.dofs[i] + d] += w * E[3 * c.id + d];
    }
}

// CG1 field at a particle: Ei = sum_i coeffs[i] * values[j*4 + i], values the
// cell's vertex values of component j (pusher.h:178-186, 318-326).
static void cg1_field(const Cell &cell, const double *Ev, const double *x, double *Ei) {
    double coeffs[4];
    cell.barycentric(x, coeffs);
    for (int j = 0; j < 3; j++) {
        Ei[j] = 0.0;
        for (int i = 0; i < 4; ++i) Ei[j] += coeffs[i] * Ev[3 * cell.dofs[i] + j];
    }
}

// accel_cg1 (punc/include/punc/pusher.h:154-201); Ev: [ndof][3].
double or_accel_cg1(void *h, const double *Ev, double dt, int32_t nthreads) {
    Oracle &o = *static_cast<Oracle *>(h);
    std::vector<double> part(std::max(1, nthreads), 0.0);
    for_cells(o.nc, nthreads, [&](int64_t cb, int64_t ce, int t) {
        double KE = 0.0;
        for (int64_t cid = cb; cid < ce; ++cid) {
            Cell &cell = o.cells[cid];
            for (auto &particle : cell.particles) {
                const double m = particle.m, q = particle.q;
                double Ei[3];
                cg1_field(cell, Ev, particle.x, Ei);
                for (int j = 0; j < 3; j++) {
                    Ei[j] *= dt * (q / m);
                    KE += 0.5 * m * particle.v[j] * (particle.v[j] + Ei[j]);
                    particle.v[j] += Ei[j];
                }
            }
        }
        part[t] = KE;
    });
    double KE = 0.0;
    for (double p : part) KE += p;
    return KE;
}

// boris_cg1 (punc/include/punc/pusher.h:282-372); Ev: [ndof][3].
double or_boris_cg1(void *h, const double *Ev, const double *B, double dt, int32_t nthreads) {
    Oracle &o = *static_cast<Oracle *>(h);
    std::vector<double> part(std::max(1, nthreads), 0.0);
    for_cells(o.nc, nthreads, [&](int64_t cb, int64_t ce, int t) {
        double KE = 0.0;
        double v_minus[3], v_prime[3], v_plus[3], tt[3], s[3], Ei[3];
        for (int64_t cid = cb; cid < ce; ++cid) {
            Cell &cell = o.cells[cid];
            for (auto &particle : cell.particles) {
                const double m = particle.m, q = particle.q;
                const double *vel = particle.v;
                cg1_field(cell, Ev, particle.x, Ei);
                double t_mag2 = 0.0;
                for (int i = 0; i < 3; ++i) { tt[i] = std::tan((dt * q / (2.0 * m)) * B[i]); t_mag2 += tt[i] * tt[i]; }
                for (int i = 0; i < 3; ++i) s[i] = 2 * tt[i] / (1 + t_mag2);
                for (int i = 0; i < 3; ++i) v_minus[i] = vel[i] + 0.5 * dt * (q / m) * Ei[i];
                for (int i = 0; i < 3; i++) KE += 0.5 * m * v_minus[i] * v_minus[i];
                const double c1[3] = {v_minus[1] * tt[2] - v_minus[2] * tt[1], -v_minus[0] * tt[2] + v_minus[2] * tt[0],
                                      v_minus[0] * tt[1] - v_minus[1] * tt[0]};
                for (int i = 0; i < 3; ++i) v_prime[i] = v_minus[i] + c1[i];
                const double c2[3] = {v_prime[1] * s[2] - v_prime[2] * s[1], -v_prime[0] * s[2] + v_prime[2] * s[0],
                                      v_prime[0] * s[1] - v_prime[1] * s[0]};
                for (int i = 0; i < 3; ++i) v_plus[i] = v_minus[i] + c2[i];
                for (int i = 0; i < 3; ++i) particle.v[i] = v_plus[i] + 0.5 * dt * (q / m) * Ei[i];
            }
        }
        part[t] = KE;
    });
    double KE = 0.0;
    for (double p : part) KE += p;
    return KE;
}

// particle_potential_energy_cg1 (punc/include/punc/diagnostics.h:379-412).
double or_potential_energy(void *h, const double *phi) {
    const Oracle &o = *static_cast<Oracle *>(h);
    double PE = 0.0, coeffs[4];
    for (const Cell &cell : o.cells)
        for (const auto &particle : cell.particles) {
            cell.barycentric(particle.x, coeffs);
            double phi_x = 0.0;
            for (int i = 0; i < 4; ++i) phi_x += coeffs[i] * phi[cell.dofs[i]];
            PE += 0.5 * particle.q * phi_x;
        }
    return PE;
}

// density_cg1 (punc/include/punc/diagnostics.h:492-555).
void or_density_cg1(void *h, double weight_e, double weight_i, double *ne, double *ni) {
    const Oracle &o = *static_cast<Oracle *>(h);
    for (int64_t i = 0; i < o.ndof; ++i) ne[i] = ni[i] = 0.0;
    double cell_coords[4];
    for (const Cell &cell : o.cells) {
        double accum_e[4] = {0, 0, 0, 0}, accum_i[4] = {0, 0, 0, 0};
        for (const auto &particle : cell.particles) {
            cell.barycentric(particle.x, cell_coords);
            if (particle.q < 0) { for (int i = 0; i < 4; ++i) accum_e[i] += cell_coords[i]; }
            else { for (int i = 0; i < 4; ++i) accum_i[i] += cell_coords[i]; }
        }
        for (int i = 0; i < 4; ++i) { ne[cell.dofs[i]] += accum_e[i]; ni[cell.dofs[i]] += accum_i[i]; }
    }
    for (int64_t i = 0; i < o.ndof; ++i) {
        ne[i] *= o.dv_inv[i] * weight_e;
        ni[i] *= o.dv_inv[i] * weight_i;
    }
}

// density_dg0 (punc/include/punc/diagnostics.h:433-465).
void or_density_dg0(void *h, double weight_e, double weight_i, double *ne, double *ni) {
    const Oracle &o = *static_cast<Oracle *>(h);
    for (const Cell &cell : o.cells) {
        double accum_e = 0.0, accum_i = 0.0;
        for (const auto &particle : cell.particles) {
            if (particle.q > 0) accum_i += weight_i;
            else accum_e += weight_e;
        }
        ne[cell.id] = accum_e / cell.volume;
        ni[cell.id] = accum_i / cell.volume;
    }
}

// Population::statistics (punc/include/punc/population.h:746-805): Welford.
void or_statistics(void *h, double *stats) {
    const Oracle &o = *static_cast<Oracle *>(h);
    std::size_t m = 0, n = 0;
    double m_e_old = 0, m_i_old = 0;
    for (int k = 0; k < 4; ++k) stats[k] = 0.0;
    for (const Cell &cell : o.cells)
        for (const auto &particle : cell.particles) {
            double v = 0;
            for (int i = 0; i < 3; ++i) v += particle.v[i] * particle.v[i];
            v = std::sqrt(v);
            if (particle.q < 0) {
                m++;
                if (m == 1) { m_e_old = v; stats[0] = v; stats[1] = 0.0; }
                else {
                    stats[0] = m_e_old + (v - m_e_old) / m;
                    stats[1] += (v - m_e_old) * (v - stats[0]);
                    m_e_old = stats[0];
                }
            }
            if (particle.q > 0) {
                n++;
                if (n == 1) { m_i_old = v; stats[2] = v; stats[3] = 0.0; }
                else {
                    stats[2] = m_i_old + (v - m_i_old) / n;
                    stats[3] += (v - m_i_old) * (v - stats[2]);
                    m_i_old = stats[2];
                }
            }
        }
    if (m > 0) stats[1] = std::sqrt(stats[1] / (m - 1));
    if (n > 0) stats[3] = std::sqrt(stats[3] / (n - 1));
}

// Population::save_file (punc/include/punc/population.h:806-837).
int32_t or_save_population(void *h, const char *fname, int32_t binary) {
    const Oracle &o = *static_cast<Oracle *>(h);
    std::FILE *fout = std::fopen(fname, binary ? "wb" : "w");
    if (!fout) return 1;
    for (const Cell &cell : o.cells)
        for (const auto &particle : cell.particles) {
            if (binary) {
                const double rec[8] = {particle.x[0], particle.x[1], particle.x[2], particle.v[0],
                                       particle.v[1], particle.v[2], particle.q,    particle.m};
                std::fwrite(rec, sizeof(rec), 1, fout);
            } else {
                for (int i = 0; i < 3; ++i) std::fprintf(fout, "%.17g\t", particle.x[i]);
                for (int i = 0; i < 3; ++i) std::fprintf(fout, "%.17g\t", particle.v[i]);
                std::fprintf(fout, "%.17g\t %.17g\t", particle.q, particle.m);
                std::fprintf(fout, "\n");
            }
        }
    std::fclose(fout);
    return 0;
}

// move / move_periodic (punc/include/punc/pusher.h:648-681).
void or_move(void *h, double dt, const double *Ld, int32_t nthreads) {
    Oracle &o = *static_cast<Oracle *>(h);
    for_cells(o.nc, nthreads, [&](int64_t cb, int64_t ce, int) {
        for (int64_t cid = cb; cid < ce; ++cid)
            for (auto &particle : o.cells[cid].particles)
                for (int j = 0; j < 3; ++j) {
                    particle.x[j] += dt * particle.v[j];
                    if (Ld) particle.x[j] -= Ld[j] * std::floor(particle.x[j] / Ld[j]);
                }
    });
}

// Population::update (punc/include/punc/population.h:641-699).  objects:
// [n][4] = {bnd_id, charge, current, potential}.  With nthreads > 1 the walks
// of a cell range run in parallel first; the bookkeeping that follows is the
// reference's sequential pass, so the result is the same.  absorbed (may be
// NULL): [tag] count of absorbed particles.  Returns 0, or -1 on a walk that
// exceeded the step limit.
int32_t or_update(void *h, double *objects, int32_t n_obj, double dt, int32_t nthreads, int64_t *absorbed,
                  int32_t n_tags) {
    Oracle &o = *static_cast<Oracle *>(h);
    for (int k = 0; k < n_obj; ++k) objects[4 * k + 2] = 0;
    std::vector<std::vector<long>> pre;
    if (nthreads > 1) {
        pre.resize(o.nc);
        for_cells(o.nc, nthreads, [&](int64_t cb, int64_t ce, int) {
            for (int64_t cid = cb; cid < ce; ++cid) {
                auto &ps = o.cells[cid].particles;
                pre[cid].resize(ps.size());
                for (size_t k = 0; k < ps.size(); ++k) pre[cid][k] = relocate_fast(o, ps[k].x, (long)cid);
            }
        });
    }
    long new_cell_id;
    for (long cell_id = 0; cell_id < (long)o.nc; ++cell_id) {
        std::vector<std::size_t> to_delete;
        std::size_t num_particles = o.cells[cell_id].particles.size();
        for (std::size_t p_id = 0; p_id < num_particles; ++p_id) {
            auto particle = o.cells[cell_id].particles[p_id];
            // a particle appended by a lower cell was already walked to here
            if (nthreads > 1 && p_id < pre[cell_id].size()) new_cell_id = pre[cell_id][p_id];
            else new_cell_id = relocate_fast(o, particle.x, cell_id);
            if (new_cell_id == LONG_MIN) return -1;
            if (new_cell_id != cell_id) {
                to_delete.push_back(p_id);
                if (new_cell_id >= 0) {
                    o.cells[new_cell_id].particles.push_back(particle);
                } else {
                    if (absorbed && -new_cell_id < n_tags) absorbed[-new_cell_id]++;
                    for (int k = 0; k < n_obj; ++k)
                        if ((std::size_t)(-new_cell_id) == (std::size_t)objects[4 * k]) objects[4 * k + 2] += particle.q;
                }
            }
        }
        std::size_t size_to_delete = to_delete.size();
        for (std::size_t it = size_to_delete; it-- > 0;) {
            auto p_id = to_delete[it];
            o.cells[cell_id].particles[p_id] = o.cells[cell_id].particles.back();
            o.cells[cell_id].particles.pop_back();
        }
    }
    for (int k = 0; k < n_obj; ++k) {
        objects[4 * k + 1] += objects[4 * k + 2];
        objects[4 * k + 2] /= dt;
    }
    return 0;
}

// distribute_cg1 (punc/include/punc/distributor.h:168-210).
void or_distribute_cg1(void *h, double *rho, int32_t nthreads) {
    Oracle &o = *static_cast<Oracle *>(h);
    const int nt = std::max(1, nthreads);
    std::vector<std::vector<double>> part(nt, std::vector<double>(o.ndof, 0.0));
    for_cells(o.nc, nt, [&](int64_t cb, int64_t ce, int t) {
        std::vector<double> &rho0 = part[t];
        double cell_coords[4];
        for (int64_t cid = cb; cid < ce; ++cid) {
            const Cell &cell = o.cells[cid];
            double accum[4] = {0.0, 0.0, 0.0, 0.0};
            for (auto &particle : cell.particles) {
                cell.barycentric(particle.x, cell_coords);
                for (int i = 0; i < 4; ++i) accum[i] += particle.q * cell_coords[i];
            }
            for (int i = 0; i < 4; ++i) rho0[cell.dofs[i]] += accum[i];
        }
    });
    for (int64_t i = 0; i < o.ndof; ++i) {
        double s = part[0][i];
        for (int t = 1; t < nt; ++t) s += part[t][i];
        rho[i] = s * o.dv_inv[i];
    }
}

// kinetic_energy (punc/include/punc/diagnostics.h:248-265).
double or_kinetic_energy(void *h) {
    const Oracle &o = *static_cast<Oracle *>(h);
    double KE = 0.0;
    for (auto &cell : o.cells)
        for (auto &particle : cell.particles)
            for (int i = 0; i < 3; ++i) KE += 0.5 * particle.m * particle.v[i] * particle.v[i];
    return KE;
}

// Image charge per object: sum over object facets of eps0*area*(grad phi . n)
// (Charge.ufl ds-integral used by CircuitCM::post_solve, punc/src/object_CM.cpp:328-337).
void or_image_charges(void *h, const double *phi, int32_t n_obj, double *out) {
    const Oracle &o = *static_cast<Oracle *>(h);
    for (int k = 0; k < n_obj; ++k) out[k] = 0.0;
    for (size_t f = 0; f < o.ofac.size() / 7; ++f) {
        const double *r = &o.ofac[7 * f];
        const Cell &c = o.cells[(int64_t)r[0]];
        const double *A = c.barycentric_matrix;
        const double p3 = phi[c.dofs[3]];
        const double a = phi[c.dofs[0]] - p3, b = phi[c.dofs[1]] - p3, e = phi[c.dofs[2]] - p3;
        double g[3];
        for (int d = 0; d < 3; ++d) g[d] = a * A[1 + d] + b * A[5 + d] + e * A[9 + d];
        const int k = (int)r[1];
        if (k >= 0 && k < n_obj) out[k] += (o.eps0 * r[2]) * (g[0] * r[3] + g[1] * r[4] + g[2] * r[5]);
    }
}

// Jacobi-preconditioned CG on the Dirichlet-eliminated system (the same
// algorithm the engine runs), for the CPU baseline.  x holds the initial
// guess and receives the solution.  Returns the iteration count, or -1.
int32_t or_pcg(void *h, const double *b_in, const int64_t *kind, const double *gval, double *x, double rtol,
               double atol, int32_t max_iter, int32_t remove_mean, int32_t nthreads) {
    const Oracle &o = *static_cast<Oracle *>(h);
    const int64_t n = o.ndof;
    std::vector<double> b(b_in, b_in + n), r(n), z(n), p(n, 0.0), Ap(n), dinv(n, 1.0);
    const int nt = std::max(1, nthreads);
    auto matvec = [&](const std::vector<double> &v, std::vector<double> &out) {
        for_cells(n, nt, [&](int64_t rb, int64_t re, int) {
            for (int64_t i = rb; i < re; ++i) {
                if (kind[i] >= 0) { out[i] = v[i]; continue; }
                double s = 0.0;
                for (int64_t k = o.rowptr[i]; k < o.rowptr[i + 1]; ++k)
                    if (kind[o.col[k]] < 0) s += o.K[k] * v[o.col[k]];
                out[i] = s;
            }
        });
    };
    for (int64_t i = 0; i < n; ++i) {
        if (kind[i] >= 0) { x[i] = gval[i]; continue; }
        for (int64_t k = o.rowptr[i]; k < o.rowptr[i + 1]; ++k)
            if (o.col[k] == i) dinv[i] = 1.0 / o.K[k];
    }
    if (remove_mean) {
        double s = 0.0;
        for (double v : b) s += v;
        for (double &v : b) v -= s / n;
    }
    std::vector<double> xv(x, x + n);
    matvec(xv, Ap);
    double rz = 0, rr = 0, bb = 0;
    for (int64_t i = 0; i < n; ++i) { r[i] = b[i] - Ap[i]; z[i] = dinv[i] * r[i]; rz += r[i] * z[i]; rr += r[i] * r[i]; bb += b[i] * b[i]; }
    const double tol = std::max(rtol * std::sqrt(bb), atol);
    int it = 0;
    double beta = 0.0;
    while (std::sqrt(rr) > tol && it < max_iter) {
        ++it;
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        matvec(p, Ap);
        double pap = 0;
        for (int64_t i = 0; i < n; ++i) pap += p[i] * Ap[i];
        if (!(pap > 0)) return -1;
        const double alpha = rz / pap;
        double rzn = 0;
        rr = 0;
        for (int64_t i = 0; i < n; ++i) { xv[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; z[i] = dinv[i] * r[i]; rzn += r[i] * z[i]; rr += r[i] * r[i]; }
        beta = rzn / rz;
        rz = rzn;
    }
    if (remove_mean) {
        double s = 0.0;
        for (double v : xv) s += v;
        for (double &v : xv) v -= s / n;
    }
    std::copy(xv.begin(), xv.end(), x);
    return std::sqrt(rr) <= tol ? it : -1;
}

// ---- AMG-preconditioned CG for the timed CPU baseline ---------------------
// The reference solves the Poisson system with PETSc's GMRES preconditioned by
// hypre's algebraic multigrid (punc/src/poisson.cpp:297-304).  The CPU
// baseline keeps that solver class with a textbook smoothed-aggregation AMG
// (Vanek, Mandel, Brezina 1996) under CG on the symmetric Dirichlet-eliminated
// system: aggregates of strongly coupled neighbourhoods (|a_ij| >= theta
// sqrt(a_ii a_jj), theta = 0.08 halved per level), tentative prolongator P0
// (one per aggregate), smoothed
// P = (I - w D^-1 A) P0 with w = 4 / (3 lambda_max(D^-1 A)), Galerkin coarse
// operators P^T A P down to at most 400 rows, a dense Cholesky solve on the
// coarsest level (a periodic system's constant null space regularised away),
// and one weighted-Jacobi sweep (weight w of the level) before and after each
// coarse correction (a symmetric V-cycle).  Products run on nthreads threads.

struct Csr {
    int64_t n = 0, m = 0;                 // rows, columns
    std::vector<int64_t> ptr, col;
    std::vector<double> val;
};

static void csr_matvec(const Csr &A, const double *x, double *y, int nt) {
    for_cells(A.n, nt, [&](int64_t rb, int64_t re, int) {
        for (int64_t i = rb; i < re; ++i) {
            double s = 0.0;
            for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) s += A.val[k] * x[A.col[k]];
            y[i] = s;
        }
    });
}

static Csr csr_transpose(const Csr &A) {
    Csr T;
    T.n = A.m; T.m = A.n;
    T.ptr.assign(T.n + 1, 0);
    for (int64_t c : A.col) ++T.ptr[c + 1];
    for (int64_t i = 0; i < T.n; ++i) T.ptr[i + 1] += T.ptr[i];
    T.col.resize(A.col.size());
    T.val.resize(A.val.size());
    std::vector<int64_t> pos(T.ptr.begin(), T.ptr.end() - 1);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int64_t q = pos[A.col[k]]++;
            T.col[q] = i;
            T.val[q] = A.val[k];
        }
    return T;
}

// C = A B (Gustavson's row-by-row product with a dense accumulator per thread).
static Csr csr_matmul(const Csr &A, const Csr &B, int nt) {
    Csr C;
    C.n = A.n; C.m = B.m;
    const int T = std::max(1, nt);
    std::vector<std::vector<int64_t>> rcol(A.n);
    std::vector<std::vector<double>> rval(A.n);
    for_cells(A.n, T, [&](int64_t rb, int64_t re, int) {
        std::vector<double> acc(B.m, 0.0);
        std::vector<int64_t> mark(B.m, -1), used;
        for (int64_t i = rb; i < re; ++i) {
            used.clear();
            for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
                const int64_t j = A.col[k];
                const double a = A.val[k];
                for (int64_t q = B.ptr[j]; q < B.ptr[j + 1]; ++q) {
                    const int64_t c = B.col[q];
                    if (mark[c] != i) { mark[c] = i; acc[c] = 0.0; used.push_back(c); }
                    acc[c] += a * B.val[q];
                }
            }
            std::sort(used.begin(), used.end());
            rcol[i] = used;
            rval[i].resize(used.size());
            for (size_t t = 0; t < used.size(); ++t) rval[i][t] = acc[used[t]];
        }
    });
    C.ptr.assign(C.n + 1, 0);
    for (int64_t i = 0; i < C.n; ++i) C.ptr[i + 1] = C.ptr[i] + (int64_t)rcol[i].size();
    C.col.resize(C.ptr[C.n]);
    C.val.resize(C.ptr[C.n]);
    for (int64_t i = 0; i < C.n; ++i) {
        std::copy(rcol[i].begin(), rcol[i].end(), C.col.begin() + C.ptr[i]);
        std::copy(rval[i].begin(), rval[i].end(), C.val.begin() + C.ptr[i]);
    }
    return C;
}

struct AmgLevel {
    Csr A, P, R;                 // operator, prolongator to this level from the next, R = P^T
    std::vector<double> dinv;
    double omega = 2.0 / 3.0;    // smoother weight 4 / (3 lambda_max(D^-1 A))
    std::vector<double> x, b, r; // work vectors
};

struct OracleAmg {
    std::vector<AmgLevel> lev;
    std::vector<double> chol;    // dense Cholesky factor of the coarsest operator (row-major, lower)
    int64_t nc = 0;
    std::vector<int64_t> free_of; // reduced index -> dof
    std::vector<int64_t> red_of;  // dof -> reduced index or -1
    int periodic = 0;
};

static std::vector<int64_t> aggregate(const Csr &A, const std::vector<double> &diag, double theta, int64_t &n_agg) {
    const int64_t n = A.n;
    std::vector<int64_t> agg(n, -1);
    auto strong = [&](int64_t i, int64_t k) {
        const int64_t j = A.col[k];
        return j != i && std::fabs(A.val[k]) >= theta * std::sqrt(std::fabs(diag[i] * diag[j]));
    };
    n_agg = 0;
    // pass 1: nodes whose strong neighbourhood is still free seed an aggregate
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool ok = true;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1] && ok; ++k)
            if (strong(i, k) && agg[A.col[k]] >= 0) ok = false;
        if (!ok) continue;
        agg[i] = n_agg;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (strong(i, k)) agg[A.col[k]] = n_agg;
        ++n_agg;
    }
    // pass 2: the rest join the aggregate they couple to most strongly
    std::vector<int64_t> first(agg);
    for (int64_t i = 0; i < n; ++i) {
        if (first[i] >= 0) continue;
        double best = -1.0;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int64_t j = A.col[k];
            if (strong(i, k) && first[j] >= 0 && std::fabs(A.val[k]) > best) { best = std::fabs(A.val[k]); agg[i] = first[j]; }
        }
    }
    // pass 3: leftovers (no strongly coupled aggregate) form their own
    for (int64_t i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        agg[i] = n_agg;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (strong(i, k) && agg[A.col[k]] < 0) agg[A.col[k]] = n_agg;
        ++n_agg;
    }
    return agg;
}

static void amg_vcycle(const OracleAmg &M, std::vector<AmgLevel> &lev, size_t l, int nt) {
    AmgLevel &L = lev[l];
    const int64_t n = L.A.n;
    if (l + 1 == lev.size()) {
        // dense Cholesky solve of the coarsest system
        std::vector<double> y(L.b);
        for (int64_t i = 0; i < n; ++i) {
            double s = y[i];
            for (int64_t k = 0; k < i; ++k) s -= M.chol[i * n + k] * y[k];
            y[i] = s / M.chol[i * n + i];
        }
        for (int64_t i = n - 1; i >= 0; --i) {
            double s = y[i];
            for (int64_t k = i + 1; k < n; ++k) s -= M.chol[k * n + i] * y[k];
            y[i] = s / M.chol[i * n + i];
        }
        L.x = y;
        return;
    }
    const double w = L.omega;
    for (int64_t i = 0; i < n; ++i) L.x[i] = w * L.dinv[i] * L.b[i];
    csr_matvec(L.A, L.x.data(), L.r.data(), nt);
    for (int64_t i = 0; i < n; ++i) L.r[i] = L.b[i] - L.r[i];
    AmgLevel &C = lev[l + 1];
    csr_matvec(L.R, L.r.data(), C.b.data(), nt);
    amg_vcycle(M, lev, l + 1, nt);
    csr_matvec(L.P, C.x.data(), L.r.data(), nt);
    for (int64_t i = 0; i < n; ++i) L.x[i] += L.r[i];
    csr_matvec(L.A, L.x.data(), L.r.data(), nt);
    for (int64_t i = 0; i < n; ++i) L.x[i] += w * L.dinv[i] * (L.b[i] - L.r[i]);
}

// AMG hierarchy of the Dirichlet-eliminated stiffness matrix (free dofs,
// kind < 0); periodic: all dofs, constant null space.  Returns a handle.
void *or_amg_setup(void *h, const int64_t *kind, int32_t periodic, int32_t nthreads) {
    const Oracle &o = *static_cast<Oracle *>(h);
    const int nt = std::max(1, nthreads);
    OracleAmg *M = new OracleAmg;
    M->periodic = periodic;
    M->red_of.assign(o.ndof, -1);
    for (int64_t i = 0; i < o.ndof; ++i)
        if (periodic || kind[i] < 0) { M->red_of[i] = (int64_t)M->free_of.size(); M->free_of.push_back(i); }
    Csr A;
    A.n = A.m = (int64_t)M->free_of.size();
    A.ptr.assign(A.n + 1, 0);
    for (int64_t r = 0; r < A.n; ++r) {
        const int64_t i = M->free_of[r];
        for (int64_t k = o.rowptr[i]; k < o.rowptr[i + 1]; ++k) {
            const int64_t c = M->red_of[o.col[k]];
            if (c >= 0 && o.K[k] != 0.0) { A.col.push_back(c); A.val.push_back(o.K[k]); }
        }
        A.ptr[r + 1] = (int64_t)A.col.size();
    }
    for (;;) {
        AmgLevel L;
        L.A = std::move(A);
        const int64_t n = L.A.n;
        std::vector<double> diag(n, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t k = L.A.ptr[i]; k < L.A.ptr[i + 1]; ++k)
                if (L.A.col[k] == i) diag[i] = L.A.val[k];
        L.dinv.resize(n);
        for (int64_t i = 0; i < n; ++i) L.dinv[i] = diag[i] != 0.0 ? 1.0 / diag[i] : 1.0;
        L.x.assign(n, 0.0); L.b.assign(n, 0.0); L.r.assign(n, 0.0);
        if (n <= 400 || M->lev.size() >= 12) { M->lev.push_back(std::move(L)); break; }
        int64_t na = 0;
        const double theta = 0.08 * std::pow(0.5, (double)M->lev.size());
        const std::vector<int64_t> agg = aggregate(L.A, diag, theta, na);
        if (na >= n) { M->lev.push_back(std::move(L)); break; }
        // lambda_max(D^-1 A) by power iteration
        std::vector<double> v(n), t(n);
        for (int64_t i = 0; i < n; ++i) v[i] = 1.0 + 0.5 * std::sin(0.7 * (double)i);
        double lam = 1.0;
        for (int it = 0; it < 20; ++it) {
            csr_matvec(L.A, v.data(), t.data(), nt);
            double num = 0.0, den = 0.0;
            for (int64_t i = 0; i < n; ++i) { t[i] *= L.dinv[i]; num += t[i] * t[i]; den += v[i] * v[i]; }
            lam = std::sqrt(num / den);
            const double s = 1.0 / std::sqrt(num);
            for (int64_t i = 0; i < n; ++i) v[i] = t[i] * s;
        }
        const double omega = 4.0 / (3.0 * lam);
        L.omega = omega;
        // P = (I - omega D^-1 A) P0
        Csr P0;
        P0.n = n; P0.m = na;
        P0.ptr.resize(n + 1);
        P0.col.resize(n);
        P0.val.assign(n, 1.0);
        for (int64_t i = 0; i < n; ++i) { P0.ptr[i] = i; P0.col[i] = agg[i]; }
        P0.ptr[n] = n;
        Csr S = L.A;
        for (int64_t i = 0; i < n; ++i)
            for (int64_t k = S.ptr[i]; k < S.ptr[i + 1]; ++k) {
                S.val[k] *= -omega * L.dinv[i];
                if (S.col[k] == i) S.val[k] += 1.0;
            }
        L.P = csr_matmul(S, P0, nt);
        L.R = csr_transpose(L.P);
        Csr AP = csr_matmul(L.A, L.P, nt);
        A = csr_matmul(L.R, AP, nt);
        M->lev.push_back(std::move(L));
    }
    // dense Cholesky of the coarsest operator (periodic: + mean(diag)/n 11^T)
    const Csr &C = M->lev.back().A;
    const int64_t n = C.n;
    M->nc = n;
    std::vector<double> D(n * n, 0.0);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = C.ptr[i]; k < C.ptr[i + 1]; ++k) D[i * n + C.col[k]] += C.val[k];
    if (periodic) {
        double tr = 0.0;
        for (int64_t i = 0; i < n; ++i) tr += D[i * n + i];
        const double d = tr / ((double)n * (double)n);
        for (double &x : D) x += d;
    }
    for (int64_t j = 0; j < n; ++j) {
        double s = D[j * n + j];
        for (int64_t k = 0; k < j; ++k) s -= D[j * n + k] * D[j * n + k];
        if (!(s > 0.0)) { delete M; return nullptr; }
        D[j * n + j] = std::sqrt(s);
        for (int64_t i = j + 1; i < n; ++i) {
            double t = D[i * n + j];
            for (int64_t k = 0; k < j; ++k) t -= D[i * n + k] * D[j * n + k];
            D[i * n + j] = t / D[j * n + j];
        }
    }
    M->chol = std::move(D);
    return M;
}

int32_t or_amg_levels(void *amg, int64_t *rows, int32_t cap) {
    const OracleAmg &M = *static_cast<OracleAmg *>(amg);
    for (int32_t l = 0; l < (int32_t)M.lev.size() && l < cap; ++l) rows[l] = M.lev[l].A.n;
    return (int32_t)M.lev.size();
}

void or_amg_free(void *amg) { delete static_cast<OracleAmg *>(amg); }

// CG preconditioned by one V-cycle of the hierarchy, with the stopping test
// and conventions of or_pcg.  Returns the iteration count, or -1.
int32_t or_amg_pcg(void *h, void *amg, const double *b_in, const int64_t *kind, const double *gval, double *x,
                   double rtol, double atol, int32_t max_iter, int32_t remove_mean, int32_t nthreads) {
    const Oracle &o = *static_cast<Oracle *>(h);
    OracleAmg &M = *static_cast<OracleAmg *>(amg);
    const int nt = std::max(1, nthreads);
    const int64_t n = o.ndof;
    std::vector<double> b(b_in, b_in + n), r(n), z(n), p(n, 0.0), Ap(n);
    std::vector<AmgLevel> &lev = M.lev;
    auto matvec = [&](const std::vector<double> &v, std::vector<double> &out) {
        for_cells(n, nt, [&](int64_t rb, int64_t re, int) {
            for (int64_t i = rb; i < re; ++i) {
                if (M.red_of[i] < 0) { out[i] = v[i]; continue; }
                double s = 0.0;
                for (int64_t k = o.rowptr[i]; k < o.rowptr[i + 1]; ++k)
                    if (M.red_of[o.col[k]] >= 0) s += o.K[k] * v[o.col[k]];
                out[i] = s;
            }
        });
    };
    auto precond = [&]() {
        const int64_t nf = (int64_t)M.free_of.size();
        for (int64_t q = 0; q < nf; ++q) lev[0].b[q] = r[M.free_of[q]];
        amg_vcycle(M, lev, 0, nt);
        for (int64_t i = 0; i < n; ++i) z[i] = M.red_of[i] < 0 ? r[i] : lev[0].x[M.red_of[i]];
        if (M.periodic) {
            double s = 0.0;
            for (double v : z) s += v;
            for (double &v : z) v -= s / n;
        }
    };
    for (int64_t i = 0; i < n; ++i)
        if (M.red_of[i] < 0) x[i] = gval[i];
    if (remove_mean) {
        double s = 0.0;
        for (double v : b) s += v;
        for (double &v : b) v -= s / n;
    }
    std::vector<double> xv(x, x + n);
    matvec(xv, Ap);
    double rr = 0, bb = 0;
    for (int64_t i = 0; i < n; ++i) { r[i] = M.red_of[i] < 0 ? 0.0 : b[i] - Ap[i]; rr += r[i] * r[i]; bb += b[i] * b[i]; }
    const double tol = std::max(rtol * std::sqrt(bb), atol);
    int it = 0;
    double rz = 0.0, beta = 0.0;
    while (std::sqrt(rr) > tol && it < max_iter) {
        precond();
        double rzn = 0.0;
        for (int64_t i = 0; i < n; ++i) rzn += r[i] * z[i];
        beta = it == 0 ? 0.0 : rzn / rz;
        rz = rzn;
        ++it;
        for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        matvec(p, Ap);
        double pap = 0;
        for (int64_t i = 0; i < n; ++i) if (M.red_of[i] >= 0) pap += p[i] * Ap[i];
        if (!(pap > 0)) return -1;
        const double alpha = rz / pap;
        rr = 0;
        for (int64_t i = 0; i < n; ++i) {
            if (M.red_of[i] < 0) continue;
            xv[i] += alpha * p[i];
            r[i] -= alpha * Ap[i];
            rr += r[i] * r[i];
        }
    }
    if (remove_mean) {
        double s = 0.0;
        for (double v : xv) s += v;
        for (double &v : xv) v -= s / n;
    }
    std::copy(xv.begin(), xv.end(), x);
    return std::sqrt(rr) <= tol ? it : -1;
}

// b = M rho (full mass matrix, no boundary conditions).
void or_mass_matvec(void *h, const double *rho, double *b) {
    const Oracle &o = *static_cast<Oracle *>(h);
    for (int64_t i = 0; i < o.ndof; ++i) {
        double s = 0.0;
        for (int64_t k = o.rowptr[i]; k < o.rowptr[i + 1]; ++k) s += o.M[k] * rho[o.col[k]];
        b[i] = s;
    }
}

// create_flux (punc/src/injector.cpp:104-171) with the analytic Maxwellian
// flux count and maximum (punc/src/distributions.cpp:23-77).  sp: [n][9] =
// {q, m, n, vth, vd0, vd1, vd2, vdf_range, unused}.
void or_create_flux(void *h, const double *sp, int32_t n_species) {
    Oracle &o = *static_cast<Oracle *>(h);
    o.flux.clear();
    for (int s = 0; s < n_species; ++s) {
        SpeciesFlux F;
        const double *r = sp + 9 * s;
        F.q = r[0]; F.m = r[1]; F.n = r[2]; F.vth = r[3];
        for (int c = 0; c < 3; ++c) F.vd[c] = r[4 + c];
        F.vdf_range = r[7] > 0 ? r[7] : 5.0;
        F.vth2 = F.vth * F.vth;
        F.factor = (1.0 / (std::pow(std::sqrt(2. * M_PI * F.vth2), 3)));
        for (int c = 0; c < 3; ++c) { F.domain[c] = F.vd[c] - F.vdf_range * F.vth; F.domain[c + 3] = F.vd[c] + F.vdf_range * F.vth; }
        for (auto &e : o.ext) {
            const double *nv = e.normal;
            double vdn = 0.0;
            for (int c = 0; c < 3; ++c) vdn += nv[c] * F.vd[c];
            const double num = e.area * (F.vth / (std::sqrt(2 * M_PI)) * std::exp(-0.5 * (vdn / F.vth) * (vdn / F.vth)) +
                                         0.5 * vdn * (1. + std::erf(vdn / (std::sqrt(2) * F.vth))));
            F.num_particles.push_back(num);
            double tmp[3];
            for (int c = 0; c < 3; ++c) tmp[c] = F.vd[c] - 0.5 * nv[c] * vdn + 0.5 * nv[c] * std::sqrt(4 * F.vth2 + vdn * vdn);
            double vn = 0.0;
            for (int c = 0; c < 3; ++c) vn += tmp[c] * nv[c];
            double v_sqrt = 0.0;
            for (int c = 0; c < 3; ++c) v_sqrt += (tmp[c] - F.vd[c]) * (tmp[c] - F.vd[c]);
            F.pdf_max.push_back((vn > 0.0) * vn * (F.factor * std::exp(-0.5 * v_sqrt / F.vth2)));
        }
        o.flux.push_back(F);
    }
}

// Two uniforms of Philox block `block` of stream (c1, c2, c3).
static void uniforms2(uint64_t seed, uint32_t block, uint32_t c1, uint32_t c2, uint32_t c3, double &a, double &b) {
    uint32_t c[4] = {block, c1, c2, c3};
    Philox::round10(c, uint32_t(seed), uint32_t(seed >> 32));
    a = Stream::res53(c[0], c[1]);
    b = Stream::res53(c[2], c[3]);
}

// inject_particles (punc/include/punc/injector.h:157-232) with counter-based
// streams in place of the unseeded mt19937_64: per (species s, facet j) a
// count stream (c1 = j, c2 = s, c3 = step) whose first uniform rounds N, and
// per particle k a stream (c1 = j, c2 = s + 8(k+1), c3 = step): block 0 the
// two uniforms of random_facet_points (punc/src/injector.cpp:78-102), block 1
// the advance fraction r, blocks 2+2i and 3+2i candidate i of the flux
// rejection sampler (punc/src/injector.cpp:51-76).  Species slot s of the flux
// table is the engine's species id s.  Returns the number kept.
int64_t or_inject(void *h, double dt, uint64_t seed, uint64_t step, int64_t *counts) {
    Oracle &o = *static_cast<Oracle *>(h);
    int64_t kept_total = 0;
    int64_t slot = 0;
    const uint32_t c3 = (uint32_t)step;
    for (size_t s = 0; s < o.flux.size(); ++s) {
        SpeciesFlux &F = o.flux[s];
        int64_t kept = 0;
        for (size_t j = 0; j < o.ext.size(); ++j) {
            const ExtFacet &e = o.ext[j];
            const double N_float = F.num_particles[j] * (F.n * dt);
            std::size_t N = static_cast<std::size_t>(N_float);
            double u0, unused;
            uniforms2(seed, 0u, (uint32_t)j, (uint32_t)s, c3, u0, unused);
            if (u0 < (N_float - N)) N += 1;
            for (std::size_t i = 0; i < N; ++i) {
                const uint32_t c2 = (uint32_t)(s + 8 * (i + 1));
                double tmp[3];
                for (uint32_t cand = 0;; ++cand) {
                    double a, b, c, u;
                    uniforms2(seed, 2u + 2u * cand, (uint32_t)j, c2, c3, a, b);
                    uniforms2(seed, 3u + 2u * cand, (uint32_t)j, c2, c3, c, u);
                    const double r3[3] = {a, b, c};
                    for (int d = 0; d < 3; ++d) tmp[d] = F.domain[d] + (F.domain[d + 3] - F.domain[d]) * r3[d];
                    double vn = 0.0;
                    for (int d = 0; d < 3; ++d) vn += tmp[d] * e.normal[d];
                    double v_sqrt = 0.0;
                    for (int d = 0; d < 3; ++d) v_sqrt += (tmp[d] - F.vd[d]) * (tmp[d] - F.vd[d]);
                    const double pdf = (vn > 0.0) * vn * (F.factor * exp_series(-0.5 * v_sqrt / F.vth2));
                    if (u * F.pdf_max[j] < pdf) break;
                }
                double r1, r2, r;
                uniforms2(seed, 0u, (uint32_t)j, c2, c3, r1, r2);
                uniforms2(seed, 1u, (uint32_t)j, c2, c3, r, unused);
                double x[3];
                for (int d = 0; d < 3; ++d) x[d] = (1.0 - r1) * e.vertices[d] + r1 * e.vertices[d + 3];
                r2 = std::sqrt(r2);
                for (int d = 0; d < 3; ++d) x[d] = r2 * x[d] + (1.0 - r2) * e.vertices[2 * 3 + d];
                for (int d = 0; d < 3; ++d) x[d] = x[d] + r * dt * tmp[d];
                const long cell = relocate_fast(o, x, (long)e.cell);
                if (cell >= 0) {
                    Particle p;
                    for (int d = 0; d < 3; ++d) { p.x[d] = x[d]; p.v[d] = tmp[d]; }
                    p.q = F.q; p.m = F.m; p.id = o.next_id + slot + (int64_t)i;
                    o.cells[cell].particles.push_back(p);
                    ++kept;
                }
            }
            slot += (int64_t)N;
        }
        if (counts) counts[s] = kept;
        kept_total += kept;
    }
    o.next_id += slot;
    return kept_total;
}

int64_t or_n_ext_facets(void *h) { return (int64_t) static_cast<Oracle *>(h)->ext.size(); }
int64_t or_ndof(void *h) { return static_cast<Oracle *>(h)->ndof; }
int64_t or_next_id(void *h) { return static_cast<Oracle *>(h)->next_id; }
void or_set_next_id(void *h, int64_t v) { static_cast<Oracle *>(h)->next_id = v; }
double or_exp_series(double x) { return exp_series(x); }
void or_philox_block(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    Philox::round10(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = c[i];
}
void or_philox_uniforms(uint64_t seed, uint32_t a, uint32_t b, uint32_t c, int64_t n, double *out) {
    Stream s(seed, a, b, c);
    for (int64_t i = 0; i < n; ++i) out[i] = s();
}

}  // extern "C"
