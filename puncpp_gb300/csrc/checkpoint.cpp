// Population files of the reference (Population::save_file / load_file,
// punc/include/punc/population.h:806-878), on the engine's particles.
//
// Binary: one 64-byte record per particle, {x[3], v[3], q, m} as doubles in
// host byte order (the reference fwrites its Particle<3> struct).  Text: per
// particle "%.17g\t" for the six coordinates, then "%.17g\t %.17g\t" for q
// and m, then a newline.  Particles are written cell by cell in cell order;
// inside a cell the engine writes them by particle id (the reference writes
// its per-cell vector, whose order depends on the history of swap-deletions;
// for a freshly loaded population both are the insertion order).  Loading
// adds the particles back through pg_add_particles, grouped by (q, m) in file
// order, as Population::add_particles does particle by particle.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pg_internal.h"
#include "punc_gpu.h"

namespace {

struct Record {
    double x[3], v[3], q, m;
};
static_assert(sizeof(Record) == 64, "the reference's Particle<3> record is 64 bytes");

}  // namespace

extern "C" int pg_population_save(pg_sim *sim, const char *fname, int32_t binary) {
    if (!sim || !fname) return pg::fail(PG_ERR_ARG, "pg_population_save: NULL argument");
    int64_t n = 0, neg = 0, pos = 0;
    int rc = pg_num_particles(sim, &n, &neg, &pos);
    if (rc) return rc;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), q(n), m(n);
    int64_t got = 0;
    rc = pg_get_particles(sim, n, x.data(), v.data(), q.data(), m.data(), nullptr, nullptr, &got);
    if (rc) return rc;
    std::FILE *f = std::fopen(fname, binary ? "wb" : "w");
    if (!f) return pg::fail(PG_ERR_ARG, std::string("pg_population_save: cannot open ") + fname);
    bool ok = true;
    for (int64_t i = 0; i < got && ok; ++i) {
        if (binary) {
            Record r;
            for (int k = 0; k < 3; ++k) { r.x[k] = x[3 * i + k]; r.v[k] = v[3 * i + k]; }
            r.q = q[i];
            r.m = m[i];
            ok = std::fwrite(&r, sizeof(r), 1, f) == 1;
        } else {
            for (int k = 0; k < 3; ++k) ok = ok && std::fprintf(f, "%.17g\t", x[3 * i + k]) > 0;
            for (int k = 0; k < 3; ++k) ok = ok && std::fprintf(f, "%.17g\t", v[3 * i + k]) > 0;
            ok = ok && std::fprintf(f, "%.17g\t %.17g\t", q[i], m[i]) > 0;
            ok = ok && std::fprintf(f, "\n") > 0;
        }
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return pg::fail(PG_ERR_ARG, std::string("pg_population_save: write failed: ") + fname);
    return PG_OK;
}

extern "C" int pg_population_load(pg_sim *sim, const char *fname, int32_t binary, int64_t *n_added) {
    if (!sim || !fname) return pg::fail(PG_ERR_ARG, "pg_population_load: NULL argument");
    std::FILE *f = std::fopen(fname, binary ? "rb" : "r");
    if (!f) return pg::fail(PG_ERR_ARG, std::string("pg_population_load: cannot open ") + fname);
    std::vector<Record> recs;
    if (binary) {
        Record r;
        while (std::fread(&r, sizeof(r), 1, f) == 1) recs.push_back(r);
    } else {
        // a line holds up to eight numbers: x, v, q, m; missing ones keep the
        // previous line's values (the reference's stream parse)
        double vals[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        std::string line;
        int ch;
        while (true) {
            line.clear();
            while ((ch = std::fgetc(f)) != EOF && ch != '\n') line.push_back((char)ch);
            if (line.empty() && ch == EOF) break;
            const char *p = line.c_str();
            int i = 0;
            while (i < 8) {
                char *end = nullptr;
                errno = 0;
                const double d = std::strtod(p, &end);
                if (end == p) break;
                vals[i++] = d;
                p = end;
            }
            Record r;
            for (int k = 0; k < 3; ++k) { r.x[k] = vals[k]; r.v[k] = vals[3 + k]; }
            r.q = vals[6];
            r.m = vals[7];
            recs.push_back(r);
            if (ch == EOF) break;
        }
    }
    std::fclose(f);
    // add in file order (the reference adds the records one by one,
    // population.h:857-878), batching each run of consecutive records with
    // the same (q, m) into one pg_add_particles call
    int64_t total = 0;
    std::vector<double> xs, vs;
    size_t i = 0;
    while (i < recs.size()) {
        const double q = recs[i].q, m = recs[i].m;
        xs.clear();
        vs.clear();
        size_t j = i;
        for (; j < recs.size() && recs[j].q == q && recs[j].m == m; ++j)
            for (int c = 0; c < 3; ++c) { xs.push_back(recs[j].x[c]); vs.push_back(recs[j].v[c]); }
        int64_t added = 0;
        const int rc = pg_add_particles(sim, xs.data(), vs.data(), (int64_t)(j - i), q, m, &added);
        if (rc) return rc;
        total += added;
        i = j;
    }
    if (n_added) *n_added = total;
    return PG_OK;
}
