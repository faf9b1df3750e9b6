// FP64 line operators: LGL nodes/weights, unit-interval mass and stiffness
// matrices, D = M^-1 S and the lift columns.  See basis.h.
#include "basis.h"

#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

namespace dg {

namespace {

// Legendre polynomials P_0..P_N at x by the three-term recurrence.
void legendre_all(int N, double x, std::vector<double>& P)
{
    P.assign(N + 1, 0.0);
    P[0] = 1.0;
    if (N >= 1) P[1] = x;
    for (int k = 2; k <= N; k++) P[k] = ((2 * k - 1) * x * P[k - 1] - (k - 1) * P[k - 2]) / k;
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n, Chebyshev start).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w)
{
    x.resize(n);
    w.resize(n);
    std::vector<double> P;
    for (int i = 0; i < n; i++) {
        double z = -std::cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            legendre_all(n, z, P);
            double dp = n * (z * P[n] - P[n - 1]) / (z * z - 1.0);
            double dz = P[n] / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        legendre_all(n, z, P);
        double dp = n * (z * P[n] - P[n - 1]) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Lagrange basis values and derivatives on nodes t at the point s.
void lagrange(const std::vector<double>& t, double s, std::vector<double>& L, std::vector<double>& dL)
{
    const int K = (int)t.size();
    L.assign(K, 1.0);
    dL.assign(K, 0.0);
    for (int j = 0; j < K; j++) {
        for (int m = 0; m < K; m++)
            if (m != j) L[j] *= (s - t[m]) / (t[j] - t[m]);
        for (int k = 0; k < K; k++) {
            if (k == j) continue;
            double term = 1.0 / (t[j] - t[k]);
            for (int m = 0; m < K; m++)
                if (m != j && m != k) term *= (s - t[m]) / (t[j] - t[m]);
            dL[j] += term;
        }
    }
}

std::string hex_of(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, 8);
    char buf[32];
    std::snprintf(buf, sizeof buf, "%016" PRIX64, b);
    return buf;
}

bool parse_hex(const std::string& s, double& v)
{
    if (s.empty() || s.size() > 16) return false;
    uint64_t b = 0;
    for (char c : s) {
        int d;
        if (c >= '0' && c <= '9') d = c - '0';
        else if (c >= 'a' && c <= 'f') d = c - 'a' + 10;
        else if (c >= 'A' && c <= 'F') d = c - 'A' + 10;
        else return false;
        b = (b << 4) | (uint64_t)d;
    }
    std::memcpy(&v, &b, 8);
    return true;
}

}  // namespace

void lgl_nodes(int K, std::vector<double>& x, std::vector<double>& w)
{
    x.assign(K, 0.0);
    w.assign(K, 0.0);
    if (K == 1) {
        w[0] = 2.0;
        return;
    }
    const int N = K - 1;
    for (int i = 0; i < K; i++) x[i] = -std::cos(M_PI * i / N);
    std::vector<double> P;
    for (int it = 0; it < 200; it++) {
        double maxd = 0;
        for (int i = 0; i < K; i++) {
            legendre_all(N, x[i], P);
            double nx = x[i] - (x[i] * P[N] - P[N - 1]) / (K * P[N]);
            maxd = std::fmax(maxd, std::fabs(nx - x[i]));
            x[i] = nx;
        }
        if (maxd < 1e-16) break;
    }
    for (int i = 0; i < K; i++) {
        legendre_all(N, x[i], P);
        w[i] = 2.0 / (N * K * P[N] * P[N]);
    }
    x[0] = -1.0;
    x[N] = 1.0;
}

void unit_matrices(int order, bool lumped, std::vector<double>& M, std::vector<double>& S)
{
    const int K = order + 1;
    std::vector<double> xi, wl, t(K), g, gw, L, dL;
    lgl_nodes(K, xi, wl);
    for (int i = 0; i < K; i++) t[i] = 0.5 * (xi[i] + 1.0);
    gauss_legendre(K + 2, g, gw);
    M.assign(K * K, 0.0);
    S.assign(K * K, 0.0);
    for (size_t q = 0; q < g.size(); q++) {
        double s = 0.5 * (g[q] + 1.0), wq = 0.5 * gw[q];
        lagrange(t, s, L, dL);
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) {
                if (!lumped) M[i * K + j] += wq * L[i] * L[j];
                S[i * K + j] += wq * dL[i] * L[j];
            }
    }
    if (lumped)
        for (int i = 0; i < K; i++) M[i * K + i] = 0.5 * wl[i];
}

bool solve_dense(int K, std::vector<double> A, std::vector<double>& B, int R)
{
    for (int c = 0; c < K; c++) {
        int piv = c;
        for (int i = c + 1; i < K; i++)
            if (std::fabs(A[i * K + c]) > std::fabs(A[piv * K + c])) piv = i;
        if (A[piv * K + c] == 0.0) return false;
        if (piv != c) {
            for (int j = 0; j < K; j++) std::swap(A[c * K + j], A[piv * K + j]);
            for (int r = 0; r < R; r++) std::swap(B[c * R + r], B[piv * R + r]);
        }
        for (int i = c + 1; i < K; i++) {
            double m = A[i * K + c] / A[c * K + c];
            for (int j = c; j < K; j++) A[i * K + j] -= m * A[c * K + j];
            for (int r = 0; r < R; r++) B[i * R + r] -= m * B[c * R + r];
        }
    }
    for (int r = 0; r < R; r++)
        for (int i = K - 1; i >= 0; i--) {
            double v = B[i * R + r];
            for (int j = i + 1; j < K; j++) v -= A[i * K + j] * B[j * R + r];
            B[i * R + r] = v / A[i * K + i];
        }
    return true;
}

namespace {

// matrices.txt reader with the reference's semantics (cppsrc/Grid.cpp:964-986):
// blocks "Order=N" followed by N+1 mass rows then N+1 stiffness rows.
std::string read_matrix_file(const std::string& path, int order, std::vector<double>& M,
                             std::vector<double>& S)
{
    std::ifstream f(path);
    if (!f.is_open())
        return "Opening file '" + path + "' failed, it either doesn't exist or is not accessible.";
    const int K = order + 1;
    M.assign(K * K, 0.0);
    S.assign(K * K, 0.0);
    std::string line;
    int cur = -1, row = 0;
    while (std::getline(f, line)) {
        if (line.compare(0, 6, "Order=") == 0) {
            cur = std::atoi(line.c_str() + 6);
            if (cur > order) break;
            continue;
        }
        if (cur != order || row >= 2 * K) continue;
        std::istringstream iss(line);
        std::string tok;
        for (int c = 0; c < K; c++) {
            double v;
            if (!(iss >> tok) || !parse_hex(tok, v)) return "malformed row in " + path;
            (row < K ? M[row * K + c] : S[(row - K) * K + c]) = v;
        }
        row++;
    }
    if (row < 2 * K) return "order " + std::to_string(order) + " not found in " + path;
    return "";
}

// hardcoded_coeff.txt reader (cppsrc/Basis.cpp:133-170): the block with index
// ``order`` (0-based) holds the zeros used by elements of that order.
std::string read_coeff_file(const std::string& path, int order, std::vector<double>& z,
                            std::vector<double>& w)
{
    std::ifstream f(path);
    if (!f.is_open())
        return "Opening file '" + path + "' failed, it either doesn't exist or is not accessible.";
    std::string line;
    int block = -1, phase = 0, npts = 0;
    while (std::getline(f, line)) {
        if (phase == 0) {
            block++;
            npts = std::atoi(line.c_str() + 2);
        } else if (block == order) {
            std::istringstream iss(line);
            std::vector<double>& dst = phase == 1 ? z : w;
            dst.clear();
            std::string tok;
            for (int i = 0; i < npts; i++) {
                double v;
                if (!(iss >> tok) || !parse_hex(tok, v)) return "malformed line in " + path;
                dst.push_back(v);
            }
            if (phase == 2) {
                if ((int)z.size() != order + 1) return "block " + std::to_string(order) + " of " + path + " has the wrong point count";
                return "";
            }
        }
        phase = (phase + 1) % 3;
    }
    return "order " + std::to_string(order) + " not found in " + path;
}

}  // namespace

std::string build_line_operators(int order, bool lumped, const std::string& matrix_file,
                                 const std::string& coeff_file, LineOperators& op)
{
    if (order < 1 || order > 9) return "order must be in 1..9";
    const int K = order + 1;
    op.order = order;
    lgl_nodes(K, op.zeros, op.weights);
    if (!coeff_file.empty()) {
        std::string err = read_coeff_file(coeff_file, order, op.zeros, op.weights);
        if (!err.empty()) return err;
    }
    if (!matrix_file.empty()) {
        std::string err = read_matrix_file(matrix_file, order, op.mass, op.stiff);
        if (!err.empty()) return err;
    } else {
        unit_matrices(order, lumped, op.mass, op.stiff);
    }
    op.deriv = op.stiff;
    if (!solve_dense(K, op.mass, op.deriv, K)) return "mass matrix is singular";
    std::vector<double> E(K * 2, 0.0);
    E[0 * 2 + 0] = 1.0;
    E[(K - 1) * 2 + 1] = 1.0;
    if (!solve_dense(K, op.mass, E, 2)) return "mass matrix is singular";
    op.lift0.resize(K);
    op.liftN.resize(K);
    for (int i = 0; i < K; i++) {
        op.lift0[i] = E[i * 2 + 0];
        op.liftN[i] = E[i * 2 + 1];
    }
    return "";
}

std::string write_coeff_files(const std::string& folder, int kmax)
{
    std::ofstream f1(folder + "/hardcoded_coeff.txt"), f2(folder + "/hardcoded_coeff2.txt");
    if (!f1.is_open() || !f2.is_open()) return "cannot write coefficient files in " + folder;
    for (int K = 1; K <= kmax; K++) {
        std::vector<double> x, w, L, dL;
        lgl_nodes(K, x, w);
        f1 << "n=" << K << "\n";
        for (int i = 0; i < K; i++) f1 << (i ? " " : "") << hex_of(x[i]);
        f1 << "\n";
        for (int i = 0; i < K; i++) f1 << (i ? " " : "") << hex_of(w[i]);
        f1 << "\n";
        f2 << "p=" << K << "\n";
        for (int i = 0; i < K; i++) {
            lagrange(x, x[i], L, dL);
            for (int j = 0; j < K; j++) f2 << (j ? " " : "") << hex_of(dL[j]);
            f2 << "\n";
        }
    }
    return "";
}

std::string write_matrix_file(const std::string& path, int max_order, bool lumped)
{
    std::ofstream f(path);
    if (!f.is_open()) return "cannot write " + path;
    for (int N = 1; N <= max_order; N++) {
        std::vector<double> M, S;
        unit_matrices(N, lumped, M, S);
        const int K = N + 1;
        f << "Order=" << N << "\n";
        for (int i = 0; i < K; i++) {
            for (int j = 0; j < K; j++) f << (j ? " " : "") << hex_of(M[i * K + j]);
            f << "\n";
        }
        for (int i = 0; i < K; i++) {
            for (int j = 0; j < K; j++) f << (j ? " " : "") << hex_of(S[i * K + j]);
            f << "\n";
        }
    }
    return "";
}

}  // namespace dg
