// Host-side check of the device-memory ledger (ledger.h): reservations up to
// the budget, refusal beyond it with nothing reserved, release, budgets below
// the bytes in use refused, and concurrent reservations that never exceed the
// budget.  Built and run by tests/test_serving_host.py; prints "ok".
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "ledger.h"

static int fails = 0;
#define CHECK(c)                                     \
  do {                                               \
    if (!(c)) {                                      \
      std::printf("FAIL line %d: %s\n", __LINE__, #c); \
      fails++;                                       \
    }                                                \
  } while (0)

int main() {
  ighost::Ledger l;
  CHECK(l.reserve(1000) && l.used() == 1000);  // no budget: anything fits
  CHECK(l.set_budget(1500) && l.budget() == 1500);
  CHECK(!l.set_budget(999));                   // below the bytes in use
  CHECK(l.reserve(500) && l.used() == 1500);   // exactly to the budget
  CHECK(!l.reserve(1) && l.used() == 1500);    // refused, nothing reserved
  CHECK(!l.reserve(UINT64_MAX) && l.used() == 1500);
  l.release(700);
  CHECK(l.used() == 800 && l.reserve(700) && !l.reserve(1));
  l.release(5000);  // over-release clamps at zero
  CHECK(l.used() == 0);
  CHECK(l.set_budget(0) && l.reserve(UINT64_MAX / 2));
  l.release(UINT64_MAX / 2);
  // concurrent reservations: the total accepted never passes the budget
  CHECK(l.set_budget(1 << 20));
  std::atomic<uint64_t> accepted{0};
  std::vector<std::thread> th;
  for (int t = 0; t < 8; t++)
    th.emplace_back([&] {
      for (int i = 0; i < 20000; i++)
        if (l.reserve(100)) accepted += 100;
    });
  for (auto& x : th) x.join();
  CHECK(accepted.load() <= (1u << 20) && accepted.load() > (1u << 20) - 100 && l.used() == accepted.load());
  if (fails) return 1;
  std::printf("ok\n");
  return 0;
}
