// Host-side check of the serving loop's dispatch decisions (serve_policy.h)
// on a 152-SM device: batch formation and the choice between the two-CTA
// cluster kernel and the one-CTA kernel, with the quarter-of-the-SMs slack
// allowed only while at most half the SMs are busy.  Built and run by
// tests/test_serving_host.py; prints "ok".
#include <cstdio>

#include "serve_policy.h"

static int fails = 0;
#define CHECK(c)                                       \
  do {                                                 \
    if (!(c)) {                                        \
      std::printf("FAIL line %d: %s\n", __LINE__, #c); \
      fails++;                                         \
    }                                                  \
  } while (0)

int main() {
  using namespace ighost;
  const size_t sms = 152, pmax = 76;
  const int64_t wait = 100000;  // 100 us
  CHECK(batch_sms(true, 8) == 16 && batch_sms(false, 8) == 8 && batch_sms(true, 0) == 0);

  // batch formation
  CHECK(launch_batch_now(128, 128, 152, sms, 0, wait));       // a full batch goes at once
  CHECK(launch_batch_now(200, 128, 400, sms, 0, wait));
  CHECK(launch_batch_now(3, 128, 151, sms, 0, wait));         // idle SMs: a partial batch goes
  CHECK(!launch_batch_now(3, 128, 152, sms, 0, wait));        // GPU full: it waits
  CHECK(!launch_batch_now(3, 128, 300, sms, wait - 1, wait));
  CHECK(launch_batch_now(3, 128, 300, sms, wait, wait));      // until its oldest query has waited
  CHECK(launch_batch_now(1, 128, 152, sms, 0, 0));            // no wait configured

  // kernel choice: an idle GPU takes any batch up to pair_max on the cluster kernel
  CHECK(use_pair_kernel(1, pmax, 0, sms));
  CHECK(use_pair_kernel(76, pmax, 0, sms));                   // 152 SMs, exactly the GPU
  CHECK(!use_pair_kernel(77, pmax, 0, sms));                  // above pair_max
  CHECK(!use_pair_kernel(1, 0, 0, sms));                      // cluster kernel off
  // at most half the SMs busy: a quarter of the SMs (38) of slack
  CHECK(!use_pair_kernel(76, pmax, 76, sms));                 // 76 + 152 = 228 > 152 + 38
  CHECK(!use_pair_kernel(58, pmax, 76, sms));                 // 76 + 116 = 192 > 190
  CHECK(use_pair_kernel(57, pmax, 76, sms));                  // 76 + 114 = 190
  CHECK(use_pair_kernel(10, pmax, 70, sms));
  // more than half busy: no slack, the batch must fit the idle SMs
  CHECK(use_pair_kernel(19, pmax, 114, sms));                 // 114 + 38 = 152
  CHECK(!use_pair_kernel(20, pmax, 114, sms));
  CHECK(!use_pair_kernel(1, pmax, 151, sms));                 // 151 + 2 > 152
  CHECK(use_pair_kernel(1, pmax, 77, sms));                   // no slack, but room
  CHECK(!use_pair_kernel(8, pmax, 1000, sms));                // oversubscribed

  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
