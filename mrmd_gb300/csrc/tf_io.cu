// Thermodynamic-force tables as text: io::dumpThermoForce and
// io::restoreThermoForce.
//
// The format is the reference's: the first line holds the bin centres, each
// further line the forces of one type, values separated by one space and
// written by std::ostream's default formatting (6 significant digits), every
// line ended by a newline.  The text side is plain host C++ (the tables are a
// few hundred bins); the device table is reached through the public
// mrmd_tf_* calls only.
#include <cmath>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"

using namespace mrmd_impl;

namespace
{
// DumpProfile::dumpScalarView (io/DumpProfile.cpp:25-35), normalisation 1.
void write_line(std::ofstream& f, const double* v, int64_t n, int64_t stride)
{
    for (int64_t i = 0; i < n; ++i)
    {
        f << v[i * stride] * 1.0;
        if (i < n - 1) f << ' ';
    }
    f << std::endl;
}

struct Table
{
    std::vector<double> grid;
    std::vector<std::vector<double>> lines;
};

// The parser of restoreThermoForce (io/RestoreThermoForce.cpp:34-73): the
// grid line's whitespace-separated values, then one force line per type,
// each value read by std::stod.
int read_table(mrmd_ctx* ctx, const char* path, int64_t maxNumForces, Table& t)
{
    std::ifstream f(path);
    if (!f) return set_error(ctx, MRMD_ERR_ARG, "cannot open thermodynamic-force table %s", path);
    std::string line, word;
    try
    {
        if (std::getline(f, line))
        {
            std::stringstream s(line);
            while (s >> word) t.grid.push_back(std::stod(word));
        }
        // MRMD_HOST_ASSERT_GREATER(binNum, 1)
        if (t.grid.size() < 2)
            return set_error(ctx, MRMD_ERR_ARG, "%s: the grid line needs at least two bins", path);
        while (std::getline(f, line))
        {
            std::vector<double> v;
            std::stringstream s(line);
            while (s >> word) v.push_back(std::stod(word));
            // The reference indexes a [grid][maxNumForces] view with these
            // counts; a line of another length has no defined result there.
            if (v.size() != t.grid.size())
                return set_error(ctx, MRMD_ERR_ARG, "%s: force line %zu has %zu values, the grid %zu", path,
                                 t.lines.size() + 1, v.size(), t.grid.size());
            t.lines.push_back(std::move(v));
            // MRMD_HOST_ASSERT_LESSEQUAL(histNum, maxNumForces)
            if ((int64_t)t.lines.size() > maxNumForces)
                return set_error(ctx, MRMD_ERR_ARG, "%s: more than %lld force lines", path,
                                 (long long)maxNumForces);
        }
    }
    catch (const std::exception&)
    {
        return set_error(ctx, MRMD_ERR_ARG, "%s: '%s' is not a number", path, word.c_str());
    }
    return MRMD_OK;
}
}  // namespace

extern "C" {

int mrmd_tf_write_table(mrmd_ctx* ctx, const char* path, int64_t numBins, const double* grid, int64_t numTypes,
                        const double* force, int64_t typeId)
{
    // io/DumpThermoForce.cpp:24-40 (one type) and :42-64 (every type)
    if (!path || !grid || !force) return set_error(ctx, MRMD_ERR_ARG, "null argument");
    if (numBins < 0 || numTypes < 1 || typeId >= numTypes)
        return set_error(ctx, MRMD_ERR_ARG, "bad table shape or type id");
    std::ofstream f(path);
    if (!f) return set_error(ctx, MRMD_ERR_ARG, "cannot write thermodynamic-force table %s", path);
    write_line(f, grid, numBins, 1);
    const int64_t first = typeId < 0 ? 0 : typeId;
    const int64_t last = typeId < 0 ? numTypes : typeId + 1;
    for (int64_t t = first; t < last; ++t) write_line(f, force + t, numBins, numTypes);
    f.close();
    if (f.fail()) return set_error(ctx, MRMD_ERR_ARG, "writing %s failed", path);
    return MRMD_OK;
}

int mrmd_tf_read_table(mrmd_ctx* ctx, const char* path, int64_t maxNumForces, int64_t* numBins,
                       int64_t* numForces, double* binWidth, double* grid, double* force, int64_t capacity)
{
    if (!path) return set_error(ctx, MRMD_ERR_ARG, "null path");
    Table t;
    MRMD_TRY(read_table(ctx, path, maxNumForces, t));
    const int64_t nb = (int64_t)t.grid.size(), nf = (int64_t)t.lines.size();
    if (numBins) *numBins = nb;
    if (numForces) *numForces = nf;
    if (binWidth) *binWidth = t.grid[1] - t.grid[0];  // RestoreThermoForce.cpp:53
    if (grid)
        for (int64_t i = 0; i < nb; ++i) grid[i] = t.grid[(size_t)i];
    if (force)
    {
        if (capacity < nb * nf) return set_error(ctx, MRMD_ERR_CAPACITY, "force buffer too small");
        for (int64_t i = 0; i < nb; ++i)
            for (int64_t k = 0; k < nf; ++k) force[i * nf + k] = t.lines[(size_t)k][(size_t)i];
    }
    return MRMD_OK;
}

int mrmd_tf_dump(mrmd_ctx* ctx, const mrmd_tf* tf, const char* path, int64_t typeId)
{
    if (!ctx || !tf || !path) return MRMD_ERR_ARG;
    int64_t nb = 0, nt = 0;
    MRMD_TRY(mrmd_tf_shape(tf, &nb, nullptr, &nt));
    std::vector<double> grid((size_t)nb), force((size_t)(nb * nt));
    MRMD_TRY(mrmd_tf_grid(tf, grid.data()));
    MRMD_TRY(mrmd_tf_get_force(ctx, tf, force.data()));
    return mrmd_tf_write_table(ctx, path, nb, grid.data(), nt, force.data(), typeId);
}

int mrmd_tf_restore(mrmd_ctx* ctx, mrmd_tf** out, const char* path, const mrmd_subdomain* sd, int64_t numTypes,
                    const double* targetDensity, const double* modulation, int enforceSymmetry, int usePeriodicity,
                    int64_t maxNumForces)
{
    // io/RestoreThermoForce.cpp:24-90
    if (!ctx || !out || !path || !sd || !targetDensity || !modulation) return MRMD_ERR_ARG;
    *out = nullptr;
    Table t;
    MRMD_TRY(read_table(ctx, path, maxNumForces, t));
    const double binWidth = t.grid[1] - t.grid[0];
    mrmd_tf* tf = nullptr;
    MRMD_TRY(mrmd_tf_create(ctx, &tf, numTypes, targetDensity, sd, binWidth, modulation, enforceSymmetry,
                            usePeriodicity));
    int64_t nb = 0;
    mrmd_tf_shape(tf, &nb, nullptr, nullptr);
    // setForce is a deep_copy, which requires equal extents
    // (ThermodynamicForce.hpp:55).
    if (nb != (int64_t)t.grid.size() || numTypes != (int64_t)t.lines.size())
    {
        mrmd_tf_destroy(ctx, tf);
        return set_error(ctx, MRMD_ERR_ARG,
                         "%s holds %zu bins x %zu types, the subdomain and types give %lld x %lld", path,
                         t.grid.size(), t.lines.size(), (long long)nb, (long long)numTypes);
    }
    std::vector<double> force((size_t)(nb * numTypes));
    for (int64_t i = 0; i < nb; ++i)
        for (int64_t k = 0; k < numTypes; ++k) force[(size_t)(i * numTypes + k)] = t.lines[(size_t)k][(size_t)i];
    const int rc = mrmd_tf_set_force(ctx, tf, force.data());
    if (rc != MRMD_OK)
    {
        mrmd_tf_destroy(ctx, tf);
        return rc;
    }
    *out = tf;
    return MRMD_OK;
}

}  // extern "C"
