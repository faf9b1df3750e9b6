// Host-side mesh construction in FP64; see mesh.h for the layout.
#include "mesh.h"

#include <cmath>
#include <cstdlib>
#include <thread>

namespace dg {

std::string validate_params(const dg_params& p)
{
    if (p.order < 1 || p.order > 7) return "ORDER must be in 1..7";  // kernels for K = 2..8 nodes per line
    for (int a = 0; a < 3; a++) {
        if (p.num_blocks[a] < 1) return "NUM_BLOCKS must be >= 1";
        if (p.num_elements[a] < 1) return "NUM_ELEMENTS must be >= 1";
        if (!(p.elem_width[a] > 0.0)) return "ELEMENT_WIDTH must be > 0";
    }
    if (!(p.rho0 > 0.0) || !(p.c0 > 0.0)) return "RHO0 and C0 must be > 0";
    for (int f = 0; f < 6; f++)
        if (p.sponge_width[f] < 0) return "BC_SPONGE_WIDTH must be >= 0";
    if (p.precision != DG_PRECISION_FP64 && p.precision != DG_PRECISION_FP32)
        return "precision must be 64 or 32";
    if (p.src_face < -1 || p.src_face > 5) return "src_face must be -1..5";
    if (p.src_face >= 0 && p.periodic[p.src_face / 2]) return "the source face must not be periodic";
    if (p.src_face >= 0 && !(p.src_freq > 0.0 && p.src_cycles > 0.0))
        return "source frequency and cycles must be > 0";
    long long ne = 1;
    for (int a = 0; a < 3; a++) ne *= (long long)p.num_blocks[a] * p.num_elements[a];
    if (ne > (1LL << 30)) return "too many elements";
    return "";
}

void MeshHost::elem_coords(int e, int g[3]) const
{
    int blk = e / elem_per_block, le = e % elem_per_block;
    int b[3] = {blk / (nb[1] * nb[2]), (blk / nb[2]) % nb[1], blk % nb[2]};
    int l[3] = {le / (ne[1] * ne[2]), (le / ne[2]) % ne[1], le % ne[2]};
    for (int a = 0; a < 3; a++) g[a] = b[a] * ne[a] + l[a];
}

int MeshHost::elem_index(const int g[3]) const
{
    int b[3], l[3];
    for (int a = 0; a < 3; a++) {
        b[a] = g[a] / ne[a];
        l[a] = g[a] % ne[a];
    }
    int blk = (b[0] * nb[1] + b[1]) * nb[2] + b[2];
    return blk * elem_per_block + (l[0] * ne[1] + l[1]) * ne[2] + l[2];
}

namespace {

// Corner of the element with global index g along axis a, computed from its
// block corner as the reference does (cppsrc/Grid.cpp:200-211 block corner,
// cppsrc/Block.cpp:172,190,208 element corner).  g may be -1 or E (halo).
double elem_corner(const dg_params& p, const MeshHost& m, int a, int g)
{
    int b = g < 0 ? 0 : (g >= m.E[a] ? m.nb[a] - 1 : g / m.ne[a]);
    int li = g - b * m.ne[a] + 1;  // local index including the halo ring
    double bc = p.corner[a] + p.elem_width[a] * m.ne[a] * b;
    return (li - 1) * p.elem_width[a] + bc;
}

// cppsrc/Element.cpp:175-177
inline double node_coord(const dg_params& p, const LineOperators& op, int a, double ec, int i)
{
    return p.elem_width[a] * (op.zeros[i] / 2.0 + .5) + ec;
}

// cppsrc/Node.cpp:76-100: Gaussian IC, distance over the enabled axes.
inline double ic_gauss(const dg_params& p, const double x[3])
{
    double d2 = 0;
    for (int a = 0; a < 3; a++)
        if (p.ic_gauss[a]) d2 += (x[a] - p.ic_center[a]) * (x[a] - p.ic_center[a]);
    double d = std::sqrt(d2);
    return std::exp(-(d) * (d) / (1.0 / p.ic_sigma));
}

// Sponge sigma of the element at global position g (cppsrc/Block.cpp:160-233):
// distance to the nearest sponged face in element widths, normalised by that
// face's sponge width, sigma = sigmaMax * max(0, 1 - d).
double sponge_sigma(const dg_params& p, const MeshHost& m, const int g[3])
{
    double dist[6];
    for (int f = 0; f < 6; f++) dist[f] = 1000000000.0;
    for (int a = 0; a < 3; a++) {
        if (p.sponge_width[2 * a] > 0) dist[2 * a] = std::abs(g[a]) * p.elem_width[a];
        if (p.sponge_width[2 * a + 1] > 0)
            dist[2 * a + 1] = std::abs(m.E[a] - std::abs(g[a]) - 1) * p.elem_width[a];
    }
    int edge = 0;
    double sh = dist[0];
    for (int f = 1; f < 6; f++)
        if (dist[f] < sh) {
            edge = f;
            sh = dist[f];
        }
    sh /= (double)p.sponge_width[edge] * p.elem_width[edge / 2];
    if (p.sponge_width[edge] == 0) return 0.0;
    return std::fmax(0.0, 1.0 - sh) * p.sigma_max;
}

}  // namespace

void MeshHost::node_coords(const dg_params& p, const LineOperators& op, int e, std::vector<double>& x) const
{
    int g[3];
    elem_coords(e, g);
    const int K3 = K * K * K;
    x.resize(3 * K3);
    double ec[3];
    for (int a = 0; a < 3; a++) ec[a] = elem_corner(p, *this, a, g[a]);
    for (int n = 0; n < K3; n++) {
        int c[3] = {n / (K * K), (n / K) % K, n % K};
        for (int a = 0; a < 3; a++) x[a * K3 + n] = node_coord(p, op, a, ec[a], c[a]);
    }
}

size_t grid_offset(const MeshHost& m, int e, int n)
{
    int g[3];
    m.elem_coords(e, g);
    const int K = m.K;
    size_t ii = (size_t)g[0] * K + n / (K * K);
    size_t jj = (size_t)g[1] * K + (n / K) % K;
    size_t kk = (size_t)g[2] * K + n % K;
    return (ii * ((size_t)m.E[1] * K) + jj) * ((size_t)m.E[2] * K) + kk;
}

std::string build_mesh(const dg_params& p, const LineOperators& op, MeshHost& m, bool with_zero_state0)
{
    std::string err = validate_params(p);
    if (!err.empty()) return err;
    m.N = p.order;
    m.K = p.order + 1;
    const int K = m.K, K2 = K * K, K3 = K * K * K;
    m.NP = (K3 + 7) / 8 * 8;
    for (int a = 0; a < 3; a++) {
        m.nb[a] = p.num_blocks[a];
        m.ne[a] = p.num_elements[a];
        m.E[a] = m.nb[a] * m.ne[a];
    }
    m.elem_per_block = m.ne[0] * m.ne[1] * m.ne[2];
    m.n_elem = m.elem_per_block * m.nb[0] * m.nb[1] * m.nb[2];
    m.nbr.assign((size_t)m.n_elem * 6, 0);
    m.sigma.assign(m.n_elem, 0.0);
    m.bnd_face.clear();

    // Neighbour table, boundary slots, sigma.
    for (int e = 0; e < m.n_elem; e++) {
        int g[3];
        m.elem_coords(e, g);
        m.sigma[e] = sponge_sigma(p, m, g);
        for (int a = 0; a < 3; a++)
            for (int side = 0; side < 2; side++) {
                int h[3] = {g[0], g[1], g[2]};
                h[a] += side ? 1 : -1;
                int f = face_of(a, side);
                if (h[a] < 0 || h[a] >= m.E[a]) {
                    if (p.periodic[a]) {
                        h[a] = (h[a] + m.E[a]) % m.E[a];
                        m.nbr[(size_t)e * 6 + f] = m.elem_index(h);
                    } else {
                        m.nbr[(size_t)e * 6 + f] = -1 - (int)m.bnd_face.size();
                        m.bnd_face.push_back(f);
                    }
                } else {
                    m.nbr[(size_t)e * 6 + f] = m.elem_index(h);
                }
            }
    }
    m.n_bnd = (int)m.bnd_face.size();

    // Boundary exterior values: IC at the halo element's face nodes, and the
    // source aperture on the source face.
    const bool ic_on = p.ic_gauss[0] || p.ic_gauss[1] || p.ic_gauss[2];
    m.bnd_ic.assign((size_t)m.n_bnd * 2 * K2, 0.0);
    m.bnd_ap.assign((size_t)m.n_bnd * K2, 0.0);
    for (int e = 0; e < m.n_elem; e++) {
        int g[3];
        m.elem_coords(e, g);
        for (int f = 0; f < 6; f++) {
            int code = m.nbr[(size_t)e * 6 + f];
            if (code >= 0) continue;
            int slot = -1 - code, a = f / 2, side = f % 2;
            int a1 = (a + 1) % 3, a2 = (a + 2) % 3;
            double ec[3];
            for (int b = 0; b < 3; b++) ec[b] = elem_corner(p, m, b, g[b]);
            ec[a] = elem_corner(p, m, a, side ? m.E[a] : -1);  // the halo element
            double ctr1 = p.corner[a1] + 0.5 * m.E[a1] * p.elem_width[a1];
            double ctr2 = p.corner[a2] + 0.5 * m.E[a2] * p.elem_width[a2];
            for (int l1 = 0; l1 < K; l1++)
                for (int l2 = 0; l2 < K; l2++) {
                    int c[3];
                    c[a] = side ? 0 : K - 1;  // the halo node touching this face
                    c[a1] = l1;
                    c[a2] = l2;
                    double x[3];
                    for (int b = 0; b < 3; b++) x[b] = node_coord(p, op, b, ec[b], c[b]);
                    size_t fi = (size_t)l1 * K + l2;
                    if (ic_on) {
                        double gs = ic_gauss(p, x);
                        m.bnd_ic[((size_t)slot * 2 + 0) * K2 + fi] = p.ic_drho_amp * gs;
                        m.bnd_ic[((size_t)slot * 2 + 1) * K2 + fi] = p.ic_v_amp[a] * gs;
                    }
                    if (f == p.src_face) {
                        double ap = 1.0;
                        if (p.src_radius > 0.0) {
                            double d1 = x[a1] - ctr1, d2 = x[a2] - ctr2;
                            if (d1 * d1 + d2 * d2 > p.src_radius * p.src_radius) ap = 0.0;
                        }
                        m.bnd_ap[(size_t)slot * K2 + fi] = ap;
                    }
                }
        }
    }

    // Initial condition in the device layout (threads over element ranges).
    if (!ic_on && !with_zero_state0) {
        m.state0.clear();
        return "";
    }
    m.state0.assign(4 * m.fstride(), 0.0);
    if (ic_on) {
        unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        if (m.n_elem < 4096) nt = 1;
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; t++)
            th.emplace_back([&, t]() {
                std::vector<double> x;
                int e0 = (int)((long long)m.n_elem * t / nt), e1 = (int)((long long)m.n_elem * (t + 1) / nt);
                for (int e = e0; e < e1; e++) {
                    m.node_coords(p, op, e, x);
                    for (int n = 0; n < K3; n++) {
                        double xn[3] = {x[n], x[K3 + n], x[2 * K3 + n]};
                        double gs = ic_gauss(p, xn);
                        size_t o = (size_t)e * m.NP + n;
                        m.state0[o] = p.ic_drho_amp * gs;
                        for (int a = 0; a < 3; a++) m.state0[(1 + a) * m.fstride() + o] = p.ic_v_amp[a] * gs;
                    }
                }
            });
        for (auto& t : th) t.join();
    }
    return "";
}

}  // namespace dg
