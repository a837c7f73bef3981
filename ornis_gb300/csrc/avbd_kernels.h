// avbd_kernels.h — host-side launchers of the AVBD device pipeline.
// Every launcher enqueues on `st` and never synchronises.
#pragma once
#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "avbd_world.cuh"

namespace avbd {

struct Tune {
    int primal_lanes = 1;        // lanes cooperating on one body in the primal (1, 4, 8, 16, 32);
                                 // 0: split primal (per (pair, side) rows, then per-body sums and solve);
                                 // -1: per-scene solve (one block takes a scene through all
                                 // iterations; split arithmetic; worlds with a scene above
                                 // SCENE_MAX_BODIES run the split launches instead)
    int primal_block = 128;      // threads per block of the primal kernel (per-scene solve: 128, 256, 512)
    int primal_minb = 4;         // resident blocks per SM the thread-per-body primal is built for
    int small_scene_max = 2048;  // scenes up to this many bodies use the one-CTA broadphase
    int sweep_rows = 1;          // larger scenes: 1 sweep per Morton-ordered cell row, 0 one x-sweep
    int fast = 0;                // 1: the fast build of the iteration kernels
    int sort_work = 0;           // 1: order each colour's bodies by incident-pair count
};

// exclusive scan of n uint32 values in place (out may alias in); tmp needs
// scan_tmp_words(n) words
size_t scan_tmp_words(size_t n);
void scan_exclusive(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp, cudaStream_t st);

// stable LSD radix sort of (key, value) pairs, n <= capacity of the buffers
void radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, size_t n,
                      uint32_t* hist, uint32_t* scan_tmp, cudaStream_t st);
size_t radix_hist_words(size_t n);
// one stable 8-bit pass (digit = (key >> shift) & 255); hist keeps the scanned
// digit-major table (digit d of tile t at hist[d * ntiles + t]); returns ntiles
int radix_pass(const uint32_t* keys, const uint32_t* vals, uint32_t* okeys, uint32_t* ovals, size_t n, int shift,
               uint32_t* hist, uint32_t* scan_tmp, cudaStream_t st);

// per substep phases
void launch_begin_substep(const DW& w, cudaStream_t st);
void launch_wake_joint_motion(const DW& w, cudaStream_t st);
void launch_gear_mem(const DW& w, cudaStream_t st);
void launch_torque(const DW& w, cudaStream_t st);
struct BroadphasePlan {
    const uint32_t* small_scenes = nullptr;  // device list of scenes swept by one CTA each
    int n_small = 0;
    std::vector<std::pair<uint32_t, uint32_t>> large;  // body ranges sorted device-wide
    uint32_t *keys_alt = nullptr, *vals_alt = nullptr, *hist = nullptr, *scan_tmp = nullptr;
    // large scenes: sweep per row of cells in Morton order (1) or one x-sweep (0)
    int rows = 1;
    uint32_t* row_key = nullptr;  // per body of the largest scene: its row's Morton code
    float* ext = nullptr;         // per large scene: the widest AABB edge
};
void launch_broadphase(const DW& w, const BroadphasePlan& plan, cudaStream_t st);
void launch_ccd(const DW& w, cudaStream_t st);
// triggers != 0: also collect this substep's trigger overlaps (an emitting substep)
void launch_discovery(const DW& w, uint32_t* scan_tmp, cudaStream_t st, int triggers = 0);
void launch_post_discovery(const DW& w, uint32_t* scan_tmp, cudaStream_t st);
void launch_colouring(const DW& w, const Tune& tune, uint32_t* scan_tmp, cudaStream_t st);

void launch_wake_apply(const DW& w, cudaStream_t st);
// Contact events of this substep (emit: the step's emitting substep) and,
// with triggers, trigger transitions; swept hits are collected every substep.
void launch_events(const DW& w, int emit, int triggers, uint32_t* scan_tmp, cudaStream_t st);
// The iteration and finish kernels exist in two builds: `exact` reproduces
// the CPU oracle bit for bit (thread-per-body primal), `fast` trades the last
// bits for fewer instructions (contracted FMAs, approximate div/sqrt).
#define AVBD_SOLVE_DECLS                                                                                    \
    void launch_iteration(const DW& w, const Tune& tune, int ncolours, cudaStream_t st);                   \
    void launch_finish_substep(const DW& w, cudaStream_t st);                                             \
    void launch_primal_colour(const DW& w, const Tune& tune, int colour, uint32_t max_bodies, cudaStream_t st); \
    void launch_dual(const DW& w, const Tune& tune, cudaStream_t st);                                   \
    void launch_solve_prep(const DW& w, const Tune& tune, cudaStream_t st);                               \
    void launch_scene_solve(const DW& w, const Tune& tune, cudaStream_t st);
namespace exact {
AVBD_SOLVE_DECLS
}
namespace fast {
AVBD_SOLVE_DECLS
}
inline void launch_iteration(const DW& w, const Tune& t, int ncol, cudaStream_t st) {
    if (t.fast) fast::launch_iteration(w, t, ncol, st);
    else exact::launch_iteration(w, t, ncol, st);
}
inline void launch_finish_substep(const DW& w, const Tune& t, cudaStream_t st) {
    if (t.fast) fast::launch_finish_substep(w, st);
    else exact::launch_finish_substep(w, st);
}
inline void launch_primal_colour(const DW& w, const Tune& t, int c, uint32_t maxb, cudaStream_t st) {
    if (t.fast) fast::launch_primal_colour(w, t, c, maxb, st);
    else exact::launch_primal_colour(w, t, c, maxb, st);
}
inline void launch_solve_prep(const DW& w, const Tune& t, cudaStream_t st) {
    if (t.fast) fast::launch_solve_prep(w, t, st);
    else exact::launch_solve_prep(w, t, st);
}
// every iteration of the substep by the per-scene solve (one launch)
inline void launch_scene_solve(const DW& w, const Tune& t, cudaStream_t st) {
    if (t.fast) fast::launch_scene_solve(w, t, st);
    else exact::launch_scene_solve(w, t, st);
}
// the per-scene solve runs when chosen and every scene fits a block
inline bool use_scene_solve(const DW& w, const Tune& t) {
    return t.primal_lanes < 0 && w.max_scene <= (uint32_t)SCENE_MAX_BODIES;
}
inline void launch_dual(const DW& w, const Tune& t, cudaStream_t st) {
    if (t.fast) fast::launch_dual(w, t, st);
    else exact::launch_dual(w, t, st);
}

// reverse of one recomputed substep (avbd_adjoint.cu)
void launch_adjoint_substep(const DW& w, const AdjFrame& f, const AdjState& A, int iters, cudaStream_t st);
void launch_adjoint_trace(const DW& w, const AdjState& A, uint2* out, cudaStream_t st);

}  // namespace avbd
