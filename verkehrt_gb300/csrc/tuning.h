// Knobs that the autotuner (verkehrt_gb300/autotune.py) picks per primitive and size class.
// Every context starts from the committed table (tuning_table.h) and may override an entry
// through vkc_tune_set, which is how the autotuner measures the candidates.
#pragma once

#include <cstdint>

#include "tuning_table.h"

namespace vkc {

enum TuneKnob {
    TK_RADIX_ITEMS = 0,       // rows per thread of the radix passes: 8, 12, 16
    TK_STREAM_BLOCKS = 1,     // blocks per SM of the streaming reductions: 2, 4, 8, 16
    TK_GATHER_ROWS = 2,       // rows per thread of gather: 1, 2, 4
    TK_GROUP_FIRST_LOG2 = 3,  // log2 of the slots of group_id's first (L2-sized) table: 18 .. 22
    TK_CHAIN_ROWS = 4,        // rows per thread and step of the canonical sums' lane chain: 4, 8, 16
    TK_COUNT = 5
};
constexpr int TUNE_CLASSES = 3;  // n < 2^20, n < 2^24, larger

struct Tuning {
    int v[TK_COUNT][TUNE_CLASSES];
};

inline int tune_class(int64_t n) { return n < (int64_t(1) << 20) ? 0 : (n < (int64_t(1) << 24) ? 1 : 2); }

inline Tuning tune_defaults() {
    Tuning t = {VKC_TUNE_TABLE};
    return t;
}

inline const char *tune_knob_name(int k) {
    static const char *names[TK_COUNT] = {"radix_items", "stream_blocks_per_sm", "gather_rows_per_thread",
                                          "group_first_table_log2", "canon_chain_rows"};
    return k >= 0 && k < TK_COUNT ? names[k] : "";
}

inline bool tune_allowed(int k, int v) {
    switch (k) {
    case TK_RADIX_ITEMS: return v == 8 || v == 12 || v == 16;
    case TK_STREAM_BLOCKS: return v == 2 || v == 4 || v == 5 || v == 6 || v == 8 || v == 12 || v == 16;
    case TK_GATHER_ROWS: return v == 1 || v == 2 || v == 4;
    case TK_GROUP_FIRST_LOG2: return v >= 18 && v <= 22;
    case TK_CHAIN_ROWS: return v == 4 || v == 8 || v == 16;
    default: return false;
    }
}

}  // namespace vkc
