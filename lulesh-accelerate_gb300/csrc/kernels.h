// kernels.h -- launchers of the step kernels (host side of the .cu files).
#pragma once

#include "lulesh_internal.h"

#include <cuda_runtime.h>

namespace lulesh {

// Threads per block of the element and node kernels.  The element kernels
// are bound by instruction issue at 64-168 registers; 128 threads give two
// to eight resident blocks per SM at their register counts (the kinematics
// kernels run two such blocks' worth as one, see kin_block).  The node
// updates, gathers bound by memory, ran 1-2 % faster in 128-thread blocks
// than in 256 (512: 2-3 % slower).
constexpr int kBlockElem = 128;
constexpr int kBlockNode = 128;

inline int elem_block(const Dom &d) { return d.eblock ? d.eblock : kBlockElem; }
inline int node_block(const Dom &d) { return d.nblock ? d.nblock : kBlockNode; }

// The kinematics kernels (128 registers, two 256-thread blocks per SM
// rather than four of 128: the same sixteen warps, but each SM sub-partition
// runs two warps of one block, which start together and walk the long
// straight-line body close to each other, so fewer warps wait on
// instruction fetch): 4-6 % faster at s=192 in both arithmetics.
constexpr int kKinBlockFactor = 2;
inline int kin_block(const Dom &d) { return kKinBlockFactor * elem_block(d); }
// Block sizes for a mesh of ne elements and nn nodes on a GPU with sms SMs:
// the defaults, halved (down to one warp) while a kernel would have fewer
// than four blocks per SM -- one FP64-bound element per thread makes the SM
// with one block more than its neighbours the one that sets the time.
inline void choose_blocks(Dom &d, int sms)
{
    int eb = kBlockElem, nb = kBlockNode;
    while (eb > 32 && (d.ne + eb - 1) / eb < 4L * sms) eb /= 2;
    while (nb > 32 && (d.nn + nb - 1) / nb < 4L * sms) nb /= 2;
    d.eblock = eb;
    d.nblock = nb;
}

// Plain FP64 path (step_fp64.cu).
void launch_time_increment(const Dom &d, cudaStream_t st);
void launch_lagrange_nodal(const Dom &d, cudaStream_t st);
void launch_lagrange_elements(const Dom &d, cudaStream_t st, bool with_constraints);
void launch_time_constraints(const Dom &d, cudaStream_t st);
void launch_finalize(const Dom &d, cudaStream_t st);
void launch_run_prologue(const Dom &d, cudaStream_t st, const int *max_cycles,
                         cudaGraphConditionalHandle h, int *active);
void launch_run_body(const Dom &d, cudaStream_t st, cudaGraphConditionalHandle h, int *active);
void launch_run_epilogue(const Dom &d, cudaStream_t st, cudaGraphConditionalHandle h, int *active);
int kernels_per_cycle();
constexpr int kRunCycleLimit = LULESH_RUN_CYCLE_BUDGET;
constexpr int kTimedKernels = 6;   // time increment, force, node, kinematics, material, finalize
void launch_cycle_timed(const Dom &d, cudaStream_t st, cudaEvent_t ev[kTimedKernels + 1]);
void launch_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t st);
void launch_rate_probe(int which, float *out, int blocks, int threads, int iters, cudaStream_t st);
// largest relative differences (as order keys of non-negative doubles) of the
// library's inverse cube root and square root from CUDA's, over n arguments
void launch_math_probe(unsigned long long *keys, int n, cudaStream_t st);

// The plain path's double-float element kernels (step_df.cu); the launchers
// above call them when Dom::df is set.
void launch_elem_force_df(const Dom &d, cudaStream_t st);
void launch_node_update_df(const Dom &d, cudaStream_t st);
void launch_elem_kinematics_df(const Dom &d, cudaStream_t st);
void launch_elem_material_df(const Dom &d, cudaStream_t st, bool with_constraints);
void launch_batch_kernel_df(const Dom &d, const BatchView &b, cudaStream_t st, int kernel, int cls, LaunchCfg cfg);
int batch_max_blocks_df(int kernel, int block);

// Split-precision path (step_split.cu).
void launch_split_sync(const Dom &d, cudaStream_t st);
void launch_lagrange_nodal_split(const Dom &d, cudaStream_t st);
void launch_lagrange_elements_split(const Dom &d, cudaStream_t st, bool with_constraints);
void launch_run_body_split(const Dom &d, cudaStream_t st, cudaGraphConditionalHandle h, int *active);
void launch_cycle_timed_split(const Dom &d, cudaStream_t st, cudaEvent_t ev[kTimedKernels + 1]);

// Batched ensembles (batch.cu drives these; kernel ids 0..3 = force, node
// update, kinematics, material).
void launch_batch_kernel_fp64(const Dom &d, const BatchView &b, cudaStream_t st, int kernel, int cls,
                              LaunchCfg cfg);
void launch_batch_kernel_split(const Dom &d, const BatchView &b, cudaStream_t st, int kernel, int cls,
                               LaunchCfg cfg);
int batch_max_blocks_fp64(int kernel, int block, int arith);
int batch_max_blocks_split(int kernel, int block);
void launch_batch_force_split_staged(const Dom &d, const BatchView &b, const StagedClass &sc, int rows,
                                     LaunchCfg cfg, cudaStream_t st);
int batch_max_blocks_split_staged(int rows);

}  // namespace lulesh
