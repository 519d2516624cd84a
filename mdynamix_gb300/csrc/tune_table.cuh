// tune_table.cuh -- written by mdynamix_gb300/autotune.py; do not edit.
// Threads per owner atom of the mixed pair sweeps, by system size (atoms)
// and mean full-row length (entries): the first cell with n <= max_atoms
// and row <= max_row wins.  Measured on NVIDIA GB300.
#pragma once

struct TuneCell {
  int max_atoms;
  double max_row;
  int tpo;
};

constexpr TuneCell TUNE_SHORT[] = {{1269, 1e30, 8}, {3549, 1e30, 8}, {12000, 1e30, 8}, {48572, 1e30, 4}, {2147483647, 1e30, 4}};
constexpr TuneCell TUNE_LONG[] = {{1269, 1e30, 32}, {3549, 1e30, 32}, {12000, 413.4, 16}, {12000, 1e30, 32}, {48572, 413.4, 8}, {48572, 1e30, 16}, {2147483647, 1e30, 8}};
