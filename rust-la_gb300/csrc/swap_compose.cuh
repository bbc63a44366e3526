// Composition of a panel's row interchanges into row moves, by one warp.
//
// A panel of jb columns starting at row j0 ends with the interchanges
// (j0 + c, x_c), c = 0 .. jb-1, applied in order (the LAPACK ipiv form that
// lu.rs:140-152 produces one column at a time). The row-swap kernel applies
// them to the columns outside the panel as one list of moves "row dst takes
// the original row src" (at most 2 jb of them). Composing the list is a
// sequential replay; done by one thread it costs one dependent memory access
// per slot scanned (thousands per panel). Here the 32 lanes of a warp search
// the slot table together with ballots, so each interchange costs a few warp
// instructions.
//
// Slots live in shared memory (at_pos / at_row, capacity SWAP_SLOTS): slot t
// says that position at_pos[t] currently holds original row at_row[t];
// positions without a slot hold their own row.
#pragma once

#include "la_internal.cuh"

constexpr int SWAP_SLOTS = 2 * MAX_PANEL_W;

// Slot whose arr[] equals val among the first na, or -1 (uniform over the warp).
__device__ __forceinline__ int swap_find(const int* arr, int na, int val, int lane) {
  for (int s = 0; s * 32 < na; s++) {
    const int t = s * 32 + lane;
    const unsigned b = __ballot_sync(0xffffffffu, t < na && arr[t] == val);
    if (b) return s * 32 + __ffs(b) - 1;
  }
  return -1;
}

// Called by all 32 lanes of one warp. by_row = false: fin[c] is x_c, the
// position swapped with j0 + c. by_row = true: fin[c] is the ORIGINAL row that
// must end at position j0 + c; x_c is its position at step c, written to
// ipiv[j0 + c] when ipiv is non-null. Writes the moves to swaps: swaps[0] =
// count, swaps[1 + i] = dst, swaps[1 + 2 MAX_PANEL_W + i] = src.
__device__ __forceinline__ void compose_swaps_warp(const int* fin, int jb, int j0, bool by_row,
                                                   int* ipiv, int* swaps, int* at_pos,
                                                   int* at_row, int lane) {
  int na = 0;
  for (int c = 0; c < jb; c++) {
    const int a = j0 + c;
    int x = fin[c];
    if (by_row) {
      const int t = swap_find(at_row, na, x, lane);
      if (t >= 0) x = at_pos[t];
    }
    if (ipiv != nullptr && lane == 0) ipiv[a] = x;
    if (x == a) continue;
    int ia = swap_find(at_pos, na, a, lane);
    int ix = swap_find(at_pos, na, x, lane);
    if (ia < 0) {
      if (lane == 0) { at_pos[na] = a; at_row[na] = a; }
      ia = na++;
    }
    if (ix < 0) {
      if (lane == 0) { at_pos[na] = x; at_row[na] = x; }
      ix = na++;
    }
    __syncwarp();
    if (lane == 0) {
      const int t = at_row[ia];
      at_row[ia] = at_row[ix];
      at_row[ix] = t;
    }
    __syncwarp();
  }
  int k = 0;
  for (int s = 0; s * 32 < na; s++) {
    const int t = s * 32 + lane;
    const bool keep = t < na && at_pos[t] != at_row[t];
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      const int o = k + __popc(b & ((1u << lane) - 1u));
      swaps[1 + o] = at_pos[t];
      swaps[1 + 2 * MAX_PANEL_W + o] = at_row[t];
    }
    k += __popc(b);
  }
  if (lane == 0) swaps[0] = k;
}
