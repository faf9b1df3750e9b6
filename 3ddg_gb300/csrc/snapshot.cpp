// Snapshot output in the reference's file layout (cppsrc/HDF5Functions.cpp:34-247):
// one file per dataset under <folder>/raw/, named <stem>_<rank>_<ts>.h5, each
// with the dataset and a one-element "time".  Every block is written as the
// MPI rank of the same number would write it (rank order = block order,
// cppsrc/Grid.cpp:292-317), with its node-duplicated local arrays.
#include <sys/stat.h>
#include <sys/types.h>

#include <string>
#include <vector>

#include "dg3d.h"
#include "h5lite.h"
#include "solver_internal.h"

namespace {

std::string fname(const std::string& folder, const char* stem, int rank, int ts)
{
    return folder + "/raw/" + stem + "_" + std::to_string(rank) + "_" + std::to_string(ts) + ".h5";
}

// Copy block b's part of a global [F][X][Y][Z] array into [F][Xb][Yb][Zb].
void block_slice(const dg::MeshHost& m, const double* g, int nf, int b, std::vector<double>& out)
{
    const int K = m.K;
    const size_t X = (size_t)m.E[0] * K, Y = (size_t)m.E[1] * K, Z = (size_t)m.E[2] * K;
    const size_t Xb = (size_t)m.ne[0] * K, Yb = (size_t)m.ne[1] * K, Zb = (size_t)m.ne[2] * K;
    const int bx = b / (m.nb[1] * m.nb[2]), by = (b / m.nb[2]) % m.nb[1], bz = b % m.nb[2];
    out.resize((size_t)nf * Xb * Yb * Zb);
    for (int f = 0; f < nf; f++)
        for (size_t i = 0; i < Xb; i++)
            for (size_t j = 0; j < Yb; j++) {
                const double* src = g + (size_t)f * X * Y * Z + ((bx * Xb + i) * Y + (by * Yb + j)) * Z + bz * Zb;
                double* dst = out.data() + (size_t)f * Xb * Yb * Zb + (i * Yb + j) * Zb;
                for (size_t k = 0; k < Zb; k++) dst[k] = src[k];
            }
}

// Place a block's [F][Xb][Yb][Zb] array into its part of the global [F][X][Y][Z].
void block_place(const dg::MeshHost& m, const double* in, int nf, int b, double* g)
{
    const int K = m.K;
    const size_t X = (size_t)m.E[0] * K, Y = (size_t)m.E[1] * K, Z = (size_t)m.E[2] * K;
    const size_t Xb = (size_t)m.ne[0] * K, Yb = (size_t)m.ne[1] * K, Zb = (size_t)m.ne[2] * K;
    const int bx = b / (m.nb[1] * m.nb[2]), by = (b / m.nb[2]) % m.nb[1], bz = b % m.nb[2];
    for (int f = 0; f < nf; f++)
        for (size_t i = 0; i < Xb; i++)
            for (size_t j = 0; j < Yb; j++) {
                const double* src = in + (size_t)f * Xb * Yb * Zb + (i * Yb + j) * Zb;
                double* dst = g + (size_t)f * X * Y * Z + ((bx * Xb + i) * Y + (by * Yb + j)) * Z + bz * Zb;
                for (size_t k = 0; k < Zb; k++) dst[k] = src[k];
            }
}

// Read dataset ``name`` of ``path``, requiring the given shape.
int read_exact(const std::string& path, const char* name, const std::vector<uint64_t>& want,
               std::vector<double>& out)
{
    std::vector<uint64_t> dims;
    std::string why;
    int rc = dg::h5_read(path, name, dims, out, nullptr, &why);
    if (rc) return dg::fail(rc, path + ": " + why);
    if (dims != want) return dg::fail(-3, path + ": dataset '" + name + "' does not have the grid's shape");
    return DG_OK;
}

}  // namespace

extern "C" int dg_hdf5_read(const char* path, const char* name, int max_ndim, long long* dims, int* ndim,
                            double* data, long long capacity, int* type_class)
{
    if (!path || !name || max_ndim < 0 || (max_ndim > 0 && !dims) || capacity < 0)
        return dg::fail(DG_ERR_INVALID, "dg_hdf5_read: bad argument");
    std::vector<uint64_t> d;
    std::vector<double> v;
    std::string why;
    int rc = dg::h5_read(path, name, d, v, type_class, &why);
    if (rc) return dg::fail(rc, std::string(path) + ": " + why);
    if (ndim) *ndim = (int)d.size();
    for (int i = 0; i < max_ndim && i < (int)d.size(); i++) dims[i] = (long long)d[i];
    if (data) {
        if ((long long)v.size() > capacity)
            return dg::fail(-3, "dg_hdf5_read: dataset holds " + std::to_string(v.size()) +
                                    " values, more than the buffer's " + std::to_string(capacity));
        std::copy(v.begin(), v.end(), data);
    }
    return DG_OK;
}

extern "C" int dg_read_snapshot(dg_handle* h, const char* folder, int ts)
{
    if (!h || !folder) return dg::fail(DG_ERR_INVALID, "dg_read_snapshot: bad argument");
    dg::Solver& s = h->s;
    const dg::MeshHost& m = s.mesh;
    const std::string dir(folder);
    const size_t gs = s.gsize();
    std::vector<double> state(4 * gs), a, v, tm;
    const uint64_t Xb = (uint64_t)m.ne[0] * m.K, Yb = (uint64_t)m.ne[1] * m.K, Zb = (uint64_t)m.ne[2] * m.K;
    const int nblocks = m.nb[0] * m.nb[1] * m.nb[2];
    double t = 0.0;
    for (int b = 0; b < nblocks; b++) {
        int rc = read_exact(fname(dir, "dRho", b, ts), "rho", {Xb, Yb, Zb}, a);
        if (!rc) rc = read_exact(fname(dir, "vel", b, ts), "velocity", {3, Xb, Yb, Zb}, v);
        if (!rc) rc = read_exact(fname(dir, "dRho", b, ts), "time", {1}, tm);
        if (rc) return rc;
        if (b == 0) t = tm[0];
        if (tm[0] != t) return dg::fail(-3, "dg_read_snapshot: the blocks' files hold different times");
        block_place(m, a.data(), 1, b, state.data());
        block_place(m, v.data(), 3, b, state.data() + gs);
    }
    int rc = dg_set_state(h, state.data(), state.data() + gs);
    if (rc) return rc;
    s.t = t;
    return DG_OK;
}

extern "C" int dg_hdf5_write(const char* path, const char* name, int ndim, const long long* dims,
                             const double* data, double time)
{
    if (!path || !name || !dims || !data || ndim < 1 || ndim > 8)
        return dg::fail(DG_ERR_INVALID, "dg_hdf5_write: bad argument");
    std::vector<uint64_t> d;
    for (int i = 0; i < ndim; i++) {
        if (dims[i] < 1) return dg::fail(DG_ERR_INVALID, "dg_hdf5_write: dimensions must be >= 1");
        d.push_back((uint64_t)dims[i]);
    }
    if (std::string(name) == "time") return dg::fail(DG_ERR_INVALID, "dg_hdf5_write: name 'time' is reserved");
    if (dg::h5_write(path, {{name, d, data}, {"time", {1}, &time}}))
        return dg::fail(-1, "HDF5 FileIException error");
    return DG_OK;
}

extern "C" int dg_write_snapshot(dg_handle* h, const char* folder, int ts, int grid)
{
    if (!h || !folder || grid < 0 || grid > 2) return dg::fail(DG_ERR_INVALID, "dg_write_snapshot: bad argument");
    dg::Solver& s = h->s;
    const dg::MeshHost& m = s.mesh;
    const std::string dir(folder);
    mkdir(dir.c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH);
    mkdir((dir + "/raw").c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH);
    const size_t gs = s.gsize();
    std::vector<double> state;
    if (grid != 2) {
        state.resize(4 * gs);
        int rc = s.pack_out(s.state_ptr(), state.data(), state.data() + gs);
        if (rc) return rc;
    }
    std::vector<double> coords, sigma;
    if (grid) {
        coords.resize(3 * gs);
        int r2 = dg_get_grid(h, coords.data(), nullptr);
        if (r2) return r2;
    }
    const int nblocks = m.nb[0] * m.nb[1] * m.nb[2];
    const uint64_t Xb = (uint64_t)m.ne[0] * m.K, Yb = (uint64_t)m.ne[1] * m.K, Zb = (uint64_t)m.ne[2] * m.K;
    const double tm = s.t;
    std::vector<double> a, v, c, cst;
    for (int b = 0; b < nblocks; b++) {
        if (grid != 2) {
            block_slice(m, state.data(), 1, b, a);
            block_slice(m, state.data() + gs, 3, b, v);
            if (dg::h5_write(fname(dir, "dRho", b, ts), {{"rho", {Xb, Yb, Zb}, a.data()}, {"time", {1}, &tm}}))
                return dg::fail(-1, "HDF5 FileIException error");
            if (dg::h5_write(fname(dir, "vel", b, ts), {{"velocity", {3, Xb, Yb, Zb}, v.data()}, {"time", {1}, &tm}}))
                return dg::fail(-1, "HDF5 FileIException error");
        }
        if (grid) {
            block_slice(m, coords.data(), 3, b, c);
            if (dg::h5_write(fname(dir, "coords", b, ts), {{"coords", {3, Xb, Yb, Zb}, c.data()}, {"time", {1}, &tm}}))
                return dg::fail(-1, "HDF5 FileIException error");
            const double vals[4] = {s.p.b_over_a, s.p.diff_const, s.p.rho0, s.p.c0};
            const char* stems[4] = {"ba", "diff", "rho0", "c0"};
            cst.assign(Xb * Yb * Zb, 0.0);
            for (int q = 0; q < 4; q++) {
                std::fill(cst.begin(), cst.end(), vals[q]);
                if (dg::h5_write(fname(dir, stems[q], b, ts), {{stems[q], {Xb, Yb, Zb}, cst.data()}, {"time", {1}, &tm}}))
                    return dg::fail(-1, "HDF5 FileIException error");
            }
        }
    }
    return DG_OK;
}
