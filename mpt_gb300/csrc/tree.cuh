// tree.cuh - internal (non-ABI) entry points of the device kd-tree for the
// planner unit.
#pragma once
#include "common.cuh"

extern "C" {
// 1-NN of nq device queries into device outputs, asynchronous on s
mptg_status mptg_tree_nearest_dev(mptg_tree* t, const double* dq, int nq, int* didx, double* dd, cudaStream_t s,
                                  bool count);
// k nearest (k <= 64, no radius) of nq device queries into device outputs
// [nq][k], sorted by (distance, id), asynchronous on s
mptg_status mptg_tree_nearest_k_dev(mptg_tree* t, const double* dq, int nq, int k, int* didx, double* dd,
                                    cudaStream_t s);
// device pointer to the FP64 master states [capacity][dim]
const double* mptg_tree_states_dev(const mptg_tree* t);
}
