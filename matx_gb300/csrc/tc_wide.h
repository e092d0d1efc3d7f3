// tc_wide.h — plan and launch of the 64-sample-row tensor-core pass (tc_wide.cu).
#pragma once
#include "common.cuh"

namespace gbfir {

struct TwParams {
  const void *x;
  int64_t x_bstride, N;
  const float *h;
  int64_t Lo, c;
  int32_t even, rev;
  double scale;
  void *out;
  int64_t out_bstride, out_len;
  int64_t up, down;
  int32_t Nt;         // outputs per row = 64*up/down (<= 128)
  int32_t NR;         // rows per tile = MMA N (64..128)
  int32_t Kp;         // K band, multiple of 32
  int64_t k0;         // band start relative to 64*q
  int32_t terms;      // 1 or 3
  int32_t fp16;       // 1: fp16 operands (one term), 0: bf16
  int32_t nraw;       // raw window slots (1 or 2)
  int32_t nsets;      // TMEM accumulator sets (1 or 2), each holding every part of one tile
  int32_t win;        // elements of xs per tile = 64*(NR-1) + Kp
  int32_t raw_elems;  // elements per raw slot
  int32_t xarr;       // bytes per swizzled term array (multiple of 1024)
  int32_t wcol0;      // first TMEM column of W (after the two accumulator sets)
  int32_t tmem_cols;
  int64_t rows, tiles_per_row, ntiles;
};

struct TwPlan {
  TwParams p;
  size_t smem;
  bool ok;
  char why[160];
};

TwPlan plan_tc_wide(int64_t up, int64_t down, int64_t Lo, int64_t c, int even, int rev, double scale, int64_t N_in,
                    int64_t out_len, int64_t batch, int xc, int precision);
int launch_tc_wide(TwPlan &pl, const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, bool xc,
                   const char *what, cudaStream_t s);

}  // namespace gbfir
