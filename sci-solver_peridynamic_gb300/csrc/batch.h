// batch.h -- data of the persistent multi-scene step (batch.cu / batch.cpp).
//
// Scenes keep their own device state (one Engine each).  A step of all scenes
// is two cooperative launches over a list of work items (runs of rows of one
// scene):
//   k_batch_pre  step start, rounds of { force pass ; adaptive decision ;
//                rollback restore or backup }, CG set-up (b, x0, r0)
//   k_batch_cg   CG iterations of every scene until all have converged, update
// With the learned warm start on, k_batch_pre ends with the features of every
// solving scene, one network launch over the rows of all scenes follows, and
// k_batch_ws_guess forms the learned guess, its residual and the guard before
// k_batch_cg.
// Per-scene CG scalars are reduced over the scene's items in item order, so
// the sums do not depend on which block ran which item.
#pragma once

#include "pd_kernels.h"

namespace pdgb {

// Per-scene constants of the step loop (Simulator::advance, simulator.cu:1159-1217).
struct SceneConst {
    int n;
    int item_begin, item_end;   // work items of this scene
    int integrator;             // 0 implicit Euler, 1 Newmark-beta
    int adaptive;               // Newmark, or adaptive_integration set
    int ticks_base;             // pd_time_step as configured
    int ticks_min;
    int max_substep;
    int phase_in_steps;
    double dt_base;
    double sphere_center0[3];
    double sphere_velocity[3];
    double origin[3];
};

// Per-scene step-loop state, advanced on the device.
struct SceneRun {
    int step;
    int substep;
    int ticks;
    int retries;           // rollbacks in the current step
    int active;            // force pass pending in this pass of the rollback loop
    int restore;           // 1: restore from the backup, 2: take the backup
    int solving;           // solve + update in this step
    int cg_converged;      // every CG solve so far converged (Simulator::CGConvergence)
    int error;             // 1: too many rollbacks in one step
    int last_iters;
    long long total_iters;
    long long rollbacks;
    long long broken;      // bonds broken so far (force passes that advanced)
    double last_res;
    double last_tol;
    double sim_time;
    double cs;             // clockScale
};

struct SceneDesc {
    StepParams P;   // time-dependent fields rewritten on the device each step
    DeviceState S;
    SceneConst C;
    WsState W;            // learned warm start: features point into the batch's buffer
    float4* rsave;        // learned warm start: residual of the previous-solution guess
    const float* ws_y;    // learned warm start: this scene's rows of the network output
};

struct WorkItem {
    int scene;
    int lo, hi;     // rows [lo, hi) of the scene
};

// Grid barrier and the uniform loop counters of the persistent kernels.
struct BatchSync {
    unsigned int count;
    unsigned int gen;
    int error;             // 1: a barrier wait ran out of time
    int pending[2];        // scenes still needing a force pass (alternating rounds)
    int running;           // scenes whose CG has not finished
    int pad[2];
};

struct BatchArgs {
    SceneDesc* scenes;
    SceneRun* run;
    const WorkItem* items;
    int n_items;
    int n_scenes;
    double* partials;      // three FP64 partials per item (arrays of n_items)
    unsigned int* counters;  // per-scene arrival counters (zero between reductions)
    BatchSync* sync;
    int max_rounds;        // force/decision rounds per step (rollbacks + 1)
    int max_cg_iters;      // bound of the CG loop over all scenes
    int tune_reps;         // > 0: only time the SpMV phase this many times
    int warm_start;        // 1: learned CG initial guess (mixed precision)
};

// Launchers (batch.cu).  Both kernels are cooperative launches: `grid` must
// not exceed the co-resident block count (blocks per SM x SMs).
cudaError_t launch_batch_pre(bool fp64, const BatchArgs& A, int grid, cudaStream_t st);
cudaError_t launch_batch_cg(bool fp64, int lanes, int unroll, const BatchArgs& A, int grid, cudaStream_t st);
int batch_pre_blocks_per_sm(bool fp64);
int batch_cg_blocks_per_sm(bool fp64, int lanes, int unroll);
// learned warm start (mixed precision): the guess, its residual and the guard
cudaError_t launch_batch_ws_guess(int lanes, int unroll, const BatchArgs& A, int grid, cudaStream_t st);
int batch_ws_blocks_per_sm(int lanes, int unroll);

}  // namespace pdgb
