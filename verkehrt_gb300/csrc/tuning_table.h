// The autotuner's table: written by `python -m verkehrt_gb300.autotune` from measurements on
// the GPU named below; edit by rerunning it. Rows are the knobs in TuneKnob order (radix rows
// per thread, streaming-reduction blocks per SM, gather rows per thread, log2 of the group_id
// first table's slots, rows per thread of the canonical sums' lane chain); columns are the
// size classes n < 2^20, n < 2^24, and larger.
// Measured on: NVIDIA GB300, 2026-12-04 (median of the runs in tuning_table.json).
#pragma once
#define VKC_TUNE_TABLE { {8, 12, 16}, {12, 16, 5}, {1, 2, 1}, {22, 21, 22}, {16, 8, 8} }
