// FP64 one-dimensional operators for the tensor-product LGL elements.
//
// Replaces the reference's Basis class inputs (cppsrc/Basis.cpp:74-237,
// hardcoded_coeff.txt) and the mass/stiffness matrices it reads from
// matrices.txt (cppsrc/Grid.cpp:920-989).  Both files are missing from the
// reference, so this module can generate them from LGL mathematics, and it can
// also read them back in the reference's hex format so that a run can use
// exactly the numbers a reference run used.
#pragma once

#include <string>
#include <vector>

namespace dg {

struct LineOperators {
    int order = 0;                 // N; K = N + 1 nodes per line
    std::vector<double> zeros;     // K LGL nodes on [-1, 1], ascending
    std::vector<double> weights;   // K LGL weights on [-1, 1]
    std::vector<double> mass;      // KxK row-major, unit interval [0, 1]
    std::vector<double> stiff;     // KxK row-major, S_ij = int_0^1 l_i' l_j
    // Derived on the host in FP64 (the reference refactors M*q*w on every
    // line of every call instead, cppsrc/Element.cpp:602):
    std::vector<double> deriv;     // D = M^-1 S  (KxK)
    std::vector<double> lift0;     // M^-1 e_0   (K)
    std::vector<double> liftN;     // M^-1 e_N   (K)
};

// LGL nodes (ascending) and weights for K points.
void lgl_nodes(int K, std::vector<double>& x, std::vector<double>& w);

// Unit-interval M and S for the given order; lumped=true gives the diagonal
// LGL-quadrature mass matrix instead of the exact one.
void unit_matrices(int order, bool lumped, std::vector<double>& M, std::vector<double>& S);

// Build every operator for ``order``.  matrix_file / coeff_file: when non-empty
// they are read in the reference's format (hex doubles) instead of computed.
// Returns an empty string on success, else an error message.
std::string build_line_operators(int order, bool lumped, const std::string& matrix_file,
                                 const std::string& coeff_file, LineOperators& out);

// Writers in the reference's formats: hardcoded_coeff.txt, hardcoded_coeff2.txt
// (point counts 1..kmax) and matrices.txt (orders 1..kmax-1).
std::string write_coeff_files(const std::string& folder, int kmax);
std::string write_matrix_file(const std::string& path, int max_order, bool lumped);

// Solve A X = B (A: KxK, B: KxR, row-major) in place of B; false if singular.
bool solve_dense(int K, std::vector<double> A, std::vector<double>& B, int R);

}  // namespace dg
