// Host-side mesh construction in FP64: element ordering, face-neighbour table,
// per-element sponge sigma, initial condition and boundary exterior values.
//
// Replaces the nested Grid -> Block -> Element -> Node containers of the
// reference (cppsrc/Grid.cpp:176-375, cppsrc/Block.cpp:139-267,
// cppsrc/Element.cpp:119-199, cppsrc/Node.cpp:61-100) by flat arrays laid out
// for the device:
//   element e = block * E_blk + (i * ne_y + j) * ne_z + k,
//     block = (bx * nb_y + by) * nb_z + bz      (the reference's rank order,
//     cppsrc/Grid.cpp:292-317), (i, j, k) the element within its block;
//   node n = (a * K + b) * K + c within an element (mNodes[a][b][c]);
//   field f of node n of element e at f * fstride + e * NP + n, NP = K^3
//     rounded up to a multiple of 8.
// There is no halo ring.  A face whose neighbour lies in another block reads
// that block's element directly (the on-device face gather that replaces
// Grid::communicate); a face on the domain boundary has a negative table
// entry -1 - slot naming a boundary slot, whose exterior state is zero except
// (a) the initial-condition halo values for the first stage after creation
// (the reference evaluates the IC in its halo ring, cppsrc/Block.cpp:167-247,
// and only the first stage of the first step reads them before setZero
// clears them, cppsrc/Grid.cpp:648-650) and (b) the tone-burst source face.
#pragma once

#include <cstddef>
#include <string>
#include <vector>

#include "basis.h"
#include "dg3d.h"

namespace dg {

// Faces in the sponge-width order of the parameter file: -X +X -Y +Y -Z +Z.
inline int face_of(int axis, int side) { return 2 * axis + side; }

struct MeshHost {
    int K = 0, N = 0, NP = 0;
    int nb[3] = {1, 1, 1};    // blocks per axis
    int ne[3] = {1, 1, 1};    // elements per block per axis
    int E[3] = {1, 1, 1};     // global elements per axis
    int n_elem = 0, elem_per_block = 0;
    int n_bnd = 0;
    std::vector<int> nbr;         // n_elem * 6
    std::vector<double> sigma;    // n_elem
    std::vector<int> bnd_face;    // n_bnd: face 0..5
    std::vector<double> bnd_ic;   // n_bnd * 2 * K*K: exterior drho, u_normal of the IC halo
    std::vector<double> bnd_ap;   // n_bnd * K*K: source aperture weight (0 off the source face)
    std::vector<double> state0;   // 4 * n_elem * NP: initial drho, u0, u1, u2 (empty: all zero)

    size_t fstride() const { return (size_t)n_elem * NP; }
    // global element coordinates of element e
    void elem_coords(int e, int g[3]) const;
    int elem_index(const int g[3]) const;
    // node coordinates of element e (interior) into x[3][K3] order (a,b,c)
    void node_coords(const dg_params& p, const LineOperators& op, int e, std::vector<double>& x) const;
};

std::string validate_params(const dg_params& p);
// With with_zero_state0 false, state0 is left empty when the initial
// condition is zero everywhere (no Gaussian axis enabled): the caller clears
// the state on the device instead of uploading zeros.
std::string build_mesh(const dg_params& p, const LineOperators& op, MeshHost& m, bool with_zero_state0 = true);

// Node-duplicated [X][Y][Z] position of node n of element e.
size_t grid_offset(const MeshHost& m, int e, int n);

}  // namespace dg
