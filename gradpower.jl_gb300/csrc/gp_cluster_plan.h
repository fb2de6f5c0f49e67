// Host-once plan of the sparse cluster factorisation.
//
// Every non-trivial generator cluster (machine + governor + exciter +
// stabiliser, src/clusters.jl:16-57) has a small sparse block A_k.  The
// reference factors it densely with partial pivoting (src/schur.jl:436-493,
// cuBLAS getrf on the GPU).  Here clusters with the same local pattern form a
// class; each class gets a static pivot choice (differential rows on their
// diagonal, algebraic rows matched to algebraic columns by maximum weight),
// a minimum-degree elimination order, and a straight-line program of slot
// operations that the GPU runs for 32 clusters per warp.
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/gradpower_gb300.h"
#include "gp_devices.cuh"

namespace gp {

struct ClusterPlan {
    int n_class = 0;
    int max_slots = 0;
    std::vector<int> cls_W, cls_rep;                 // per class: width, representative cluster
    std::vector<int> cluster_class;                  // per problem cluster (-1 trivial)
    std::vector<int> task_class, task_first, task_count, order;   // order: problem cluster ids
    std::vector<short> slot_of;                      // [class][1024]
    std::vector<int> prog_ptr, prog_mid, prog_sol, rhs_base, nslot, perm_col, pos3;
    std::vector<CluOp> ops;
    int64_t lu_flops = 0;                            // per scenario, all clusters (FMA count)
};

void make_cluster_plan(const gp_problem *pr, const double *z0, const double *u0, const double *p,
                       ClusterPlan &out);

// Host run of one cluster's program (the device kernel's operation order):
// yx[3*W] = (A^-1 f, A^-1 B(:,vr), A^-1 B(:,vi)) per local state, out8 = D, C y, I;
// returns max |f| over the cluster rows.  f_out[W] receives the BE residual.
double host_cluster_run(const gp_problem *pr, const ClusterPlan &pl, int cluster, const double *z,
                        const double *zold, const double *u0, const double *p, double dt, double *yx,
                        double *out8, double *f_out);

}  // namespace gp
