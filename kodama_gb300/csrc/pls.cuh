// PLS-LDA kernels (pls.cu): float32 SIMPLS + LDA cross-validation and
// train/predict, restating plscv.cpp's CPU path operation for operation.
//
// Work unit: a "slice" = one (problem, fold) pair of a cross-validation, or
// one problem of a projection (predict mode: every row trains, the rows to
// predict come from a separate standardised matrix).  One CTA per slice.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace kgb {

// Label-independent per-slice preparation (the fold cache of
// plscv.cpp:593-667): centring / scaling statistics, the standardised rows,
// the column sums of the standardised training rows and, on request, the
// fold Gram matrix.
struct PlsPrepArgs {
  int problems;          // R
  int F;                 // slices per problem (folds, or 1 in predict mode)
  int L;                 // rows per problem
  int p;                 // columns
  int center, scale;
  const float* X;        // R x L x p rows of each problem
  const int* train_off;  // S + 1 offsets into train_idx
  const int* train_idx;  // ascending training rows of each slice
  float* mean;           // S x p
  float* sdev;           // S x p
  float* Z;              // S x L x p standardised rows (all L rows, with the slice's statistics)
  float* xsum;           // S x p
  int* zexp;             // S x p: largest biased exponent (at least 1) of each column over the training rows
  float* gram;           // S x p x p (only for build_gram)
  // predict mode: standardise NV extra rows per problem with the slice's statistics
  const float* Xv;       // R x NV x p, or nullptr
  float* Zv;             // R x NV x p
  int NV;
};

int pls_prepare(const PlsPrepArgs& a, cudaStream_t st);
int pls_build_gram(const PlsPrepArgs& a, const uint8_t* want, cudaStream_t st);

struct PlsEvalArgs {
  int problems;          // R
  int F;                 // slices per problem
  int L;                 // rows per problem
  int p;                 // columns
  int C0max;             // stride of per-code arrays
  int max_components;    // SIMPLS rank limit
  int requested;         // components evaluated: min(requested, fitted rank)
  int predict_mode;      // 1: rows to predict are Zv rows 0..NV-1
  int da_mode;           // 1: PLS-DA (one-hot regression on the scores) instead of LDA
  int s_in_smem;         // 1: the label cross-product of a slice lives in shared memory
  int tiles_after_s;     // 1: some slice computes training scores during the fit (no fold Gram)
  const float* Z;        // S x L x p
  const float* xsum;     // S x p
  const int* zexp;       // S x p (PlsPrepArgs::zexp)
  const float* gram;     // S x p x p, or nullptr
  const uint8_t* use_gram;  // S (with gram != nullptr)
  const uint8_t* folds;  // R x L fold ids (CV), nullptr in predict mode
  const int* train_off;  // S + 1
  const int* train_idx;  // ascending training rows of each slice
  const int* val_off;    // S + 1 (CV)
  const int* val_idx;    // ascending validation rows of each slice (CV)
  const float* Zv;       // R x NV x p (predict mode)
  int NV;
  const float* w0;       // p: the SIMPLS start vector (std::mt19937(1), normal_distribution<float>)
  const float* logprior; // logf(max(k / nt, FLT_MIN)) tables
  const int* lp_off;     // S: table offset of the slice (index by class count k)
  const uint16_t* labels;     // R x L label codes
  const int* class_off;       // R x (C0max + 1) offsets into class_rows
  const uint16_t* class_rows; // R x L rows sorted by code, ascending within a code
  uint16_t* pred;        // CV: R x L predicted codes; predict: R x NV
  int* eval_comp;        // S: components evaluated by the slice
  int* status;           // S: 0 ok, 1 no supervised direction (degenerate fit), 2 LDA factorisation failed
  // scratch
  float* s_scr;          // S x p x C0max
  float* W;              // S x p x max_components
  float* V;              // S x p x max_components
  float* T;              // S x L x requested (training-row scores, by class-list position)
  float* Tt;             // S x L x requested (the same scores in training order)
  uint16_t* pos;         // S x L: position of each row in the slice's class list
  uint8_t* posok;        // S x L: whether the row at a class-list position trains the slice
  float* sc;             // S x L (scores path of the fit)
};

int pls_evaluate(const PlsEvalArgs& a, cudaStream_t st);
// Dynamic shared memory of the evaluation kernel; components are limited to 64.
size_t pls_eval_smem(int p, int C0max, int requested, int max_components, bool s_in_smem,
                     bool tiles_after_s);
constexpr int kPlsMaxComponents = 64;

// out[i] = x row rows[i] (p columns), i < nrows.
int pls_gather_rows(const float* x, int p, const int* rows, size_t nrows, float* out, cudaStream_t st);

// KODAMA.matrix result rows of the PLS classifier: landmark rows take the
// evolved labels, the other rows their PLS-LDA projection.
int pls_assemble_result(int problems, int n, int L, int NV, const int* land, const int* test_rows,
                        const uint16_t* clbest, const uint16_t* proj, const int* code2label, int C0max, int* res,
                        cudaStream_t st);

}  // namespace kgb
