// plan.h -- view canonicalisation ("view compiler") for the elementwise,
// gather and scatter kernels.
#pragma once

#include "common.cuh"

namespace phcu {

enum PlanMode : int32_t { MODE_EMPTY = 0, MODE_ROW = 1, MODE_TILE = 2 };

constexpr int TILE = 64;  // tile edge (elements) of the transpose path

// One planned launch: the output is operand 0, inputs follow.
struct EvalPlan {
  Space sp;
  Operand out;
  Operand in[MAXIN];
  int32_t nin;
  int32_t mode;
  int32_t vec;     // ROW: elements per thread-chunk (1, 2 or 4)
  int32_t raxis;   // TILE: axis along which staged inputs are contiguous
  uint32_t staged; // TILE: bit k set = input k goes through shared memory
  int64_t nrows;   // ROW: n / shape[rank-1]
  FastDiv lendiv;  // ROW: divide by shape[rank-1]
  // TILE geometry
  int64_t tiles_r, tiles_w, nbatch;
  FastDiv tdiv_w, tdiv_r;
};

// Builds a plan for out <- f(inputs).  All views must have the same shape up
// to size-1 axes.  Returns PHCU_OK, or an error with the message set.
int32_t make_plan(const phcu_view_t* out, const phcu_view_t* const* ins, int nin, EvalPlan* p,
                  int force_mode = -1);

// Byte extent [lo, hi) touched by a view.
void view_extent(const phcu_view_t* v, uintptr_t* lo, uintptr_t* hi);
bool views_overlap(const phcu_view_t* a, const phcu_view_t* b);
bool views_identical(const phcu_view_t* a, const phcu_view_t* b);
int32_t check_view(const phcu_view_t* v, const char* what);
// check_view for an input of an elementwise program: also accepts an index
// operand (dtype PHCU_INDEX, base ignored).
int32_t check_input_view(const phcu_view_t* v, const char* what);
inline bool is_index_view(const phcu_view_t* v) { return v && v->dtype == PHCU_INDEX; }
int64_t view_size(const phcu_view_t* v);
// A program the interpreter can run with `nin` inputs: known opcodes and
// types, operand sources that exist, valid conversion targets.
int32_t check_program(const phcu_program_t* prog, int nin);

}  // namespace phcu
