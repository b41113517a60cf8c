// Parameters of the persistent label-evolution kernel (evolve.cu).
#pragma once

#include <stdint.h>

#include "rng.cuh"

namespace kgb {

constexpr uint16_t kNoRow = 0xFFFFu;

// Per-problem layout: problem p owns rows [p*L, (p+1)*L) of every per-row
// array, p*C0max entries of per-code arrays, p*T of per-cycle arrays.
struct EvolveParams {
  int problems;
  int L;            // rows (landmarks) per problem
  int w;            // neighbour-table width k' (<= 32)
  int T;            // cycles
  int F;            // folds
  int C0max;        // stride of per-code arrays
  int G;            // groups (shared by all problems)
  int singleton;    // every group has exactly one member
  int evolutionary, guarded, absorption, adaptive;
  int pol_guidance, pol_adaptive, pol_transition, pol_stochastic, pol_diversity, pol_reject1;
  uint64_t bucket_count;   // libstdc++ bucket count after reserve(L)
  int smem_rows;           // 1 = per-row arrays in shared memory
  int smem_trans;          // 1 = class x prediction counts in shared memory
  // inputs
  const uint16_t* nb;      // problems x L x w local neighbour ids (kNoRow = none)
  const float* sc;         // problems x L x w scores -(d*d)
  const uint16_t* init;    // problems x L initial label codes
  const int* code2label;   // problems x C0max sorted distinct initial labels
  const int* ncodes;       // problems
  const uint8_t* nocollide;// problems: 1 if all labels lie in [0, bucket_count)
  const uint8_t* folds;    // problems x L
  const int* fixed;        // L (shared) or problems x L (per_problem_groups), or nullptr; value 1 = fixed
  const int* goff;         // G+1 group offsets (or problems x (L+1))
  const int* gmem;         // L group members (rows), ascending within a group (or problems x L)
  int per_problem_groups;  // 1: goff / gmem / fixed hold one block per problem, group counts in gcount
  const int* gcount;       // problems (per_problem_groups)
  const uint64_t* seeds;   // problems
  const double* psq;       // L+1: (c/L)*(c/L) as two rounded double operations
  const int* rev_off;      // problems x (L+1): reverse neighbour lists of the vote tables
  const uint16_t* rev_idx; // problems x L x w
  // outputs
  uint16_t* clbest;        // problems x L
  uint16_t* cvpredbest;    // problems x L
  double* vect_acc;        // problems x T
  double* vect_score;      // problems x T
  int* proposal_size;      // problems x T
  int* active;             // problems x T
  uint8_t* flags;          // problems x T x 3
  int* counters;           // problems x 16
  double* best;            // problems x 2 (accbest, scorebest)
  int* status;             // problems
  // scratch
  int* trans;              // problems x C0max x C0max
  int* foldcnt;            // problems x F x C0max
  uint16_t* rows_scratch;  // grid x 8 x L (when the per-row arrays do not fit in shared memory)
  uint64_t* raw_scratch;   // grid x (L/2 + 64) engine outputs of one shuffle
  // learned proposal (kNN singleton path): network packed by mlp_pack_params, or nullptr
  const uint32_t* mlp;
  int mlp_greedy;          // 1 = relabel the top-scored candidates; 0 = sample them (Gumbel top-k)
  // training snapshot of the state at the start of cycle snap_cycle (snap_feat nullptr = none)
  int snap_cycle;
  float* snap_feat;        // problems x L x 8
  uint16_t* snap_cur;      // problems x L
  uint16_t* snap_pred;     // problems x L
};

// Per-problem state of the PLS-LDA evolution kept between cycle launches.
struct PlsRunState {
  double accbest, scorebest, cur_acc, cur_score;
  int nc_cur, nc_best;
  int coarsened, absorbed;  // moves of the pending proposal
  int proposals, best_updates, accepts, st_att, st_acc, rejections;
  int co_moves, absorb_moves, tr_att, tr_acc, m1_att, m1_acc, co_att, co_acc, success;
};

struct EvolvePlsParams {
  EvolveParams base;       // counters has stride 18 here
  PlsRunState* state;      // problems
  Mt64State* rng;          // problems: the run's engine between launches
  uint16_t* cur;           // problems x L current state
  uint16_t* curpred;       // problems x L its CV predictions
  uint16_t* cl;            // problems x L labels to evaluate (proposal)
  const uint16_t* pred;    // problems x L CV predictions of cl
  int* class_off;          // problems x (C0max + 1)
  uint16_t* class_rows;    // problems x L rows of cl grouped by code
  const double* plogp;     // L + 1: (k/L) * log(k/L)
  const double* klogk;     // L + 1: k * log(k) (0 for k = 0)
  const double* logk;      // L + 1: log(k)
  double logn;             // log(L)
  int coarsening;          // auto_class_coarsening
  int pol_coarsen, pol_frag;
  int phase;               // 0: initial labels; 1: accept cycle-1 / propose cycle
  int cycle;
};

constexpr int kEvolveRowArrays = 8;
size_t evolve_smem_bytes(int L, int C0max, bool rows_in_smem, bool trans_in_smem);
int evolve_launch(const EvolveParams& p, int grid, size_t smem, void* stream);
int evolve_pls_launch(const EvolvePlsParams& q, int grid, size_t smem, void* stream);

}  // namespace kgb
