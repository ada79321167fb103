// serve_policy.h -- the serving loop's two dispatch decisions (serve.cu),
// kept free of CUDA so that a host-only check (tests/native) can exercise
// them.  Internal; not part of the public header.
#pragma once
#include <cstddef>
#include <cstdint>

namespace ighost {

// SMs a batch of n queries occupies: two per query on the two-CTA cluster
// kernel, one on the one-CTA kernel.
inline size_t batch_sms(bool pair, size_t n) { return (pair ? 2 : 1) * n; }

// Batch formation: a full batch goes at once; a partial one goes at once
// while the GPU has idle SMs, else when its oldest query has waited
// `wait_ns` (the batches in flight keep the GPU busy meanwhile).
inline bool launch_batch_now(size_t pending, size_t max_batch, size_t inflight_sm, size_t sm_count,
                             int64_t oldest_waited_ns, int64_t wait_ns) {
  return pending >= max_batch || inflight_sm < sm_count || oldest_waited_ns >= wait_ns;
}

// Kernel choice for a batch of nb queries: the two-CTA cluster kernel (two
// SMs per query, the lower latency) when the batch is at most pair_max
// queries and those SMs are idle, else one CTA per query (the higher rate per
// SM, which a loaded GPU needs: the cluster kernel alone serves at most
// ~70 % of the one-CTA rate).  While at most half the SMs are busy a cluster
// batch may exceed the idle SMs by a quarter of the SM count (an SM frees
// about every microsecond); that slack at any load let cluster batches starve
// a 75 %-load stream (measured: the achieved rate fell below the offered one,
// p99 > 100 ms).
inline bool use_pair_kernel(size_t nb, size_t pair_max, size_t inflight_sm, size_t sm_count) {
  const size_t slack = inflight_sm <= sm_count / 2 ? sm_count / 4 : 0;
  return nb <= pair_max && inflight_sm + 2 * nb <= sm_count + slack;
}

}  // namespace ighost
