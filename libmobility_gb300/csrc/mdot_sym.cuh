// Symmetric all-pairs product for the open-space translational block, FP32.
//
// Same product as mdot_kernel<float, kOpen, F only> (libMobility
// solvers/NBody/extra/NbodyRPY.cu:26-116 with OpenBoundary::dotProduct_UF,
// hydrodynamicKernels.cuh:41-57, 143-150), evaluated over unordered pairs:
// the open RPY block is symmetric (M_ij = M_ji, the same 3x3 tensor
// f I + G d d^T for d and -d), so the coefficients of a pair, which are most
// of its cost, are computed once and applied to both particles.
//
// Work decomposition (per batch of nper particles, tiles of 128 = 32 slots of
// four particles):
//   * a tile pair (I, J), I < J, is 32 rotation steps: at step k lane l pairs
//     the four particles of slot l of tile I (in registers) with the four of
//     slot (l + k) mod 32 of tile J (staged in the warp's own shared memory,
//     with the slot's accumulators beside it); no two lanes touch the same
//     slot in a step, so the j-side needs neither atomics nor reductions.  A
//     diagonal tile (I, I) is 16 steps: slot pairs at distance 1..15, then
//     the pairs inside each slot (exact formula, self pair included) together
//     with the slot pairs at distance 16 (lanes 0..15).  Steps are taken two
//     at a time, the second on another copy of the j sums, so each lane has
//     sixteen independent pair evaluations between warp synchronisations;
//   * the steps of all tile pairs, in a fixed order, are cut into equal
//     contiguous ranges, one per resident warp (host-built tables); a warp
//     walks its range pair by pair and writes, for each pair it touched, its
//     i-side and j-side sums as one partial slot each, at a place the host
//     reserved in the slot range of the tile the sums belong to;
//   * the evaluation is packed f32x2 (two particles of a slot per
//     instruction) with r^2 clamped at 4 (exact for separated pairs); steps
//     where a lane met a pair closer than 2a are flagged and, after the
//     pair's steps, those pairs get the exact near-field value;
//   * every tile owns the same number of slots (the largest any tile needs);
//     slots no warp writes stay zero from the plan's set-up, so the fold
//     reads a fixed range without a table;
//   * after a bounded grid barrier every thread of the grid folds a share of
//     the slot range of one output element with the two-sum transformation,
//     the shares are combined in a fixed tree (deterministic results), and U
//     is written (overwritten).
#pragma once
#include <cstddef>
#include <vector>

#include <cuda_runtime.h>

#include "rpy_pair.cuh"

namespace lmg {

constexpr int kSymTile = 128;     // particles per tile (32 slots of 4)
constexpr int kSymThreads = 128;  // four warps per block

struct SymPlan {
  int N = 0, nper = 0, nbatch = 0;
  int tpb = 0;          // tiles per batch
  int grid = 0;         // resident blocks launched (0: the kernel does not apply)
  int nwarps = 0;       // warps with a step range
  int rt = 1;           // threads per output element in the final fold
  int variant = 2;      // resident blocks per SM the kernel build is made for
  long long steps = 0;  // rotation steps of all tile pairs
  int cmax = 0;         // slots per tile
  size_t slots = 0;     // partial slots of 3 * kSymTile floats (tiles x cmax)
  size_t part_elems = 0;  // zero them once before the first launch
  // tables the kernel reads (uploaded by the caller):
  std::vector<int4> pairs;  // per tile pair (schedule order): tile I, tile J, first
                            // slot of the I-side sums, first slot of the J-side sums
  std::vector<int> pseg;    // per tile pair: (first warp << 8) | warps touching it
  std::vector<int4> warps;  // per warp, two entries: {first pair, first step, steps,
                            // pseg of that pair} and that pair's entry of `pairs`
  std::vector<int> tused;   // per tile: slots written (the rest of its range stays 0)
};

// Plans the launch; returns cudaErrorNotSupported when the shape does not
// suit the symmetric kernel (the caller then uses mdot_kernel).  force_warps
// > 0 caps the number of warps the steps are spread over (tests use it to
// cut tile pairs at many different steps).
cudaError_t mdot_sym_plan(int N, int nper, int num_sms, int force_warps, SymPlan &plan);

// The same without a device: `resident` blocks of the kernel fit on the GPU
// at once.
cudaError_t mdot_sym_plan_tables(int N, int nper, long long resident, int force_warps,
                                 SymPlan &plan);

// Device copies of the plan's tables.
struct SymTables {
  const int4 *pairs = nullptr;
  const int *pseg = nullptr;
  const int4 *warps = nullptr;
};

// U = M F over the batches of plan (positions pos, forces F: 3N interleaved,
// 16-byte aligned when nper is a multiple of 4 or there is one batch).  part
// holds plan.part_elems floats, zeroed before the first launch with this
// plan (launches leave the slots no warp writes at zero); *bar is the grid
// barrier's arrival count (zero before the first launch; every launch that
// completes leaves it at a multiple of its block count); *err (device
// visible) is set to 1 if a barrier wait ran out, and then *bar must be
// zeroed again.
cudaError_t mdot_sym_launch(const SymPlan &plan, const SymTables &tab, const float *pos,
                            const float *F, float *U, float inv_a, const PairConst<float> &k,
                            float *part, unsigned long long *bar, int *err,
                            cudaStream_t stream);

}  // namespace lmg
