/*
 * CPU oracle -- work counters (test infrastructure only).  Compiled in only
 * with -DNEBC7_PORT_COUNTERS (oracle/build_oracle.sh builds that variant as
 * liboracle_port_counters.so); the plain port has none of this.
 *
 * They count the reference's algorithmic integer work on an input, as the
 * port performs it step for step (the reference counts only calls, under
 * OPTION_COUNTERS: src/SnippetLevelsBuffer.h:7-11, src/Bc7CoreMode0.cpp:18):
 *
 *   err_calls / err_terms   subset-error evaluations (ComputeSubsetError*,
 *                           src/Snippet*.h, Mode4.cpp:159/494, Mode5.cpp:143)
 *                           and the (pixel, level, channel) terms they
 *                           evaluate up to their early exit;
 *   scan_calls / scan_terms candidate-list scans (LevelsBuffer,
 *                           LevelsBufferHalf) and their (window cell,
 *                           pixel) table terms;
 *   est_calls / est_terms   lower-bound scans (LevelsMinimum) and their
 *                           (cell, pixel) and (row, pixel) cut terms.
 *
 * The final index selection (ComputeSubsetTable, once per block) and the
 * bookkeeping around the searches are not counted.
 */
#pragma once

#include <stdint.h>

#ifdef NEBC7_PORT_COUNTERS
#include <atomic>

namespace nebc7_oracle {

enum WorkCounter
{
	kErrCalls, kErrTerms, kScanCalls, kScanTerms, kEstCalls, kEstTerms, kNumWorkCounters
};

extern std::atomic<uint64_t> gWork[kNumWorkCounters];

} // namespace nebc7_oracle

#define PORT_COUNT(which, n) (nebc7_oracle::gWork[nebc7_oracle::which].fetch_add(uint64_t(n), std::memory_order_relaxed))
#else
#define PORT_COUNT(which, n) ((void)0)
#endif
