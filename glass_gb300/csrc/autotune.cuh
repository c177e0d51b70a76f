// Launch-shape autotuner.
//
// A kernel family with several equivalent launch shapes (tile shapes, CTA
// counts) registers its candidates under a shape key (the problem size that
// matters for the choice).  The first eager call with a new key times every
// candidate on the caller's stream with CUDA events (one warm launch, then
// two timed launches each) and keeps the fastest; later calls, and calls
// made while the stream is being captured into a CUDA graph, reuse the kept
// choice (or the default candidate when none has been tuned yet).  The
// candidates must compute the same result (they are re-run), so only launch
// shape is tuned, never arithmetic.  The cache is per process; it is listed,
// cleared and switched on / off through the C ABI (gg_autotune_*), and
// GG_AUTOTUNE=0 in the environment starts it switched off.
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "common.cuh"

namespace gg {

// Returns the index of the candidate to launch.  `launch(i)` enqueues
// candidate i on `stream`.
int autotune_choose(const std::string& kernel, const std::string& shape, const std::vector<std::string>& names,
                    int fallback, cudaStream_t stream, const std::function<void(int)>& launch);

}  // namespace gg
