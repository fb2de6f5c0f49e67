// Host-once symbolic analysis of the reduced network matrix S.
//
// S is the Schur complement of the backward-Euler Jacobian onto the
// network voltages (and the algebraic states of static generators); its
// pattern is the bus adjacency graph with 2x2 blocks.  The analysis here
// replaces the reference's cuDSS "analysis" phase
// (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:776-819): a nested-dissection
// ordering on the bus graph, the elimination tree, supernodes, the
// multifrontal front layout and a level schedule for the GPU kernels.
#pragma once
#include <cstdint>
#include <vector>

namespace gp {

struct Symbolic {
    int n = 0;                       // scalar unknowns of S
    std::vector<int> perm;           // perm[k] = unknown eliminated k-th
    std::vector<int> iperm;          // iperm[perm[k]] = k
    int nsup = 0;
    std::vector<int> sup_start;      // [nsup+1] permuted column ranges
    std::vector<int> sup_of;         // [n] supernode of permuted column
    std::vector<int> parent;         // [nsup] parent supernode or -1
    std::vector<int> row_ptr, rows;  // below-block row structure (permuted, sorted)
    std::vector<int> level;          // [nsup] 0 for leaves
    int nlevels = 0;
    std::vector<int> level_ptr, level_sups;   // supernodes by level
    std::vector<int> child_ptr, children;     // children of each supernode (ascending)
    std::vector<int64_t> front_off;  // [nsup+1] offsets of m_s*m_s fronts
    std::vector<int64_t> uvec_off;   // [nsup+1] offsets of r_s update vectors
    // rel[relmap_ptr[c] + a] = front position in parent(c) of row structure entry a of c
    std::vector<int> relmap_ptr, relmap;
    int64_t nnz_lu = 0;              // entries of L+U (diagonal blocks counted once)
    double flops = 0.0;              // factorisation flops (dense front model)
    int max_front = 0;
    int front_m(int s) const { return sup_start[s + 1] - sup_start[s] + row_ptr[s + 1] - row_ptr[s]; }
    int front_n(int s) const { return sup_start[s + 1] - sup_start[s]; }
    int front_r(int s) const { return row_ptr[s + 1] - row_ptr[s]; }
};

// Analyse a structurally symmetric pattern given as CSR adjacency of the
// scalar unknowns (self loops allowed, ignored).  `group` maps every scalar
// unknown to a graph node (a bus); unknowns of one node stay adjacent in
// the ordering.  n_nodes is the number of nodes.
void analyse(int n, const std::vector<int> &rowptr, const std::vector<int> &colidx,
             const std::vector<int> &group, int n_nodes, Symbolic &out);

}  // namespace gp
