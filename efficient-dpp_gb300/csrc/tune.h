// tune.h — per-size-class tuning of the plain primitives (internal).
//
// A table of (primitive, element size, log2 of the length) -> variant,
// filled by edpp_autotune_plain or read from the committed table
// efficient-dpp_gb300/tuning/plain_gb300.tsv on first use.  The primitives
// consult it at call time; without an entry they take their default.
#pragma once

#include <cstddef>
#include <cstdint>

namespace edpp {

// The tuned variant for primitive `prim` (edpp_tune_primitive) with
// `elem_bytes`-byte elements at `length`: the entry of the nearest size
// class recorded for that primitive and element size, else `fallback`.
int tuned_variant(int prim, int elem_bytes, int64_t length, int fallback);

// Scan of `length` elements of `elem_bytes` bytes (4: int32, 8: int64) with
// an explicit variant of `algo` (EDPP_SCAN_LOOKBACK: tile shape, EDPP_SCAN_RTS:
// slice length of the chunked form), for the autotuner.  Same arguments and
// results as edpp_scan_exclusive_i32 / _i64.
int scan_with_variant(const void *in, void *out, int64_t length, int elem_bytes, int algo,
                      int variant, void *ws, size_t ws_bytes, void *stream);

// Candidate count of a tunable primitive.
int scan_variants(int algo);

}  // namespace edpp
