// Exhaustive check of the JSON codec's unsigned-integer paths (json_codec.h):
// every length from 1 to 16 digits through the compact-run fast path, the
// one-number fast path and the checked path, at every distance from the end
// of the buffer, plus the numbers serde_json rejects (leading zeros, signs,
// fractions, overflow).  Built and run by tests/test_wire.py; prints "ok"
// and exits 0, or names the first failing case and exits 1.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "json_codec.h"

using igjson::Json;

static int fails = 0;

static void check(bool ok, const std::string& what) {
  if (!ok && fails++ < 20) std::printf("FAIL: %s\n", what.c_str());
}

// Parse `text` (an array) with u64_array_into; true and the values on success.
static bool parse_array(const std::string& text, std::vector<uint64_t>& out) {
  Json j{text.data(), text.data() + text.size(), "", text.data()};
  out.assign(4096, 0);
  size_t n = 0;
  if (!j.u64_array_into(out.data(), out.size(), &n)) return false;
  j.ws();
  if (j.p != j.end) return false;
  out.resize(n);
  return true;
}

// A value of exactly `len` digits (no leading zero), varied by `salt`.
static uint64_t value_of_len(int len, uint64_t salt) {
  uint64_t lo = 1;
  for (int i = 1; i < len; i++) lo *= 10;
  const uint64_t span = lo * 9;  // [lo, 10 lo)
  return lo + (salt * 0x9E3779B97F4A7C15ull) % span;
}

int main() {
  // 1. each length alone, as the last element, and inside long runs, at
  //    every distance from the end of the buffer (trailing whitespace pads)
  for (int len = 1; len <= 16; len++) {
    for (uint64_t salt = 0; salt < 40; salt++) {
      const uint64_t v = value_of_len(len, salt);
      for (int pad = 0; pad < 20; pad++) {
        const std::string tail(pad, ' ');
        std::vector<uint64_t> got;
        // alone: the compact run of one element
        std::string t1 = "[" + std::to_string(v) + "]" + tail;
        check(parse_array(t1, got) && got.size() == 1 && got[0] == v, "alone " + t1);
        // last of a run of mixed lengths
        std::string t2 = "[";
        std::vector<uint64_t> want;
        for (int k = 1; k <= 16; k++) {
          const uint64_t w = value_of_len(k, salt + k);
          want.push_back(w);
          t2 += std::to_string(w) + ",";
        }
        t2 += std::to_string(v) + "]" + tail;
        want.push_back(v);
        check(parse_array(t2, got) && got == want, "run " + t2);
        // the checked path (whitespace after the comma), same values
        std::string t3 = "[7, " + std::to_string(v) + "]" + tail;
        check(parse_array(t3, got) && got.size() == 2 && got[0] == 7 && got[1] == v, "checked " + t3);
        // leading zero: rejected by every path
        std::string z = "0" + std::to_string(v);
        if (z.size() <= 16) {
          std::vector<uint64_t> g;
          check(!parse_array("[" + z + "]" + tail, g), "leading zero alone " + z);
          check(!parse_array("[1," + z + ",2]" + tail, g), "leading zero in run " + z);
          check(!parse_array("[1, " + z + "]" + tail, g), "leading zero checked " + z);
        }
      }
    }
  }
  // 2. zero itself, and numbers serde_json rejects
  std::vector<uint64_t> g;
  check(parse_array("[0]", g) && g.size() == 1 && g[0] == 0, "[0]");
  check(parse_array("[0,0,10,0]", g) && g == std::vector<uint64_t>({0, 0, 10, 0}), "[0,0,10,0]");
  check(parse_array("[ 0 , 0 ]", g) && g == std::vector<uint64_t>({0, 0}), "[ 0 , 0 ]");
  for (const char* bad : {"[00]", "[007]", "[1,00]", "[ 01]", "[-1]", "[1.5]", "[1e3]", "[+1]", "[1,]", "[,1]", "[]x",
                          "[18446744073709551616]", "[99999999999999999999]", "[184467440737095516150]"})
    check(!parse_array(bad, g), std::string("accepted ") + bad);
  check(parse_array("[18446744073709551615]", g) && g.size() == 1 && g[0] == 18446744073709551615ull, "u64 max");
  check(parse_array("[12345678901234567]", g) && g[0] == 12345678901234567ull, "17 digits");
  // 3. single numbers through u64()
  for (int len = 1; len <= 19; len++) {
    const uint64_t v = len <= 16 ? value_of_len(len, 3) : 1234567890123456789ull / (len == 19 ? 1 : len == 18 ? 10 : 100);
    const std::string t = std::to_string(v);
    Json j{t.data(), t.data() + t.size(), "", t.data()};
    uint64_t x = 0;
    check(j.u64(x) && x == v, "u64 " + t);
    const std::string z = "0" + t;
    Json jz{z.data(), z.data() + z.size(), "", z.data()};
    check(!jz.u64(x), "u64 leading zero " + z);
  }
  // 4. the writer: Out::num and Out::nums give std::to_string's digits for
  // every value up to 10^6, around every power of ten, and for 10^6 values
  // spread over the whole u64 range
  {
    uint64_t seed = 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
      seed ^= seed << 13;
      seed ^= seed >> 7;
      seed ^= seed << 17;
      return seed;
    };
    std::vector<uint64_t> vals;
    for (uint64_t v = 0; v <= 1000000; v++) vals.push_back(v);
    uint64_t p = 1;
    for (int k = 0; k < 20; k++) {
      for (uint64_t d : {p - 1, p, p + 1}) vals.push_back(d);
      if (k < 19) p *= 10;
    }
    vals.push_back(18446744073709551615ull);
    for (int k = 0; k < 1000000; k++) vals.push_back(next() >> (next() & 63));
    std::string want;
    igjson::Out o;
    for (size_t i = 0; i < vals.size(); i++) {
      o.n = 0;
      o.num(vals[i]);
      const std::string w = std::to_string(vals[i]);
      check(o.equals(w), "num " + w);
    }
    o.n = 0;
    o.nums(vals.data(), vals.size());
    for (size_t i = 0; i < vals.size(); i++) want += (i ? "," : "") + std::to_string(vals[i]);
    check(o.equals(want), "nums");
    // after other output, and finished with done(): no byte past a number
    // survives
    igjson::Out o2;
    o2.lit("[");
    o2.nums(vals.data() + 1000000, 64);
    o2.lit("]");
    std::string w2 = "[";
    for (size_t i = 0; i < 64; i++) w2 += (i ? "," : "") + std::to_string(vals[1000000 + i]);
    w2 += "]";
    check(o2.done() == w2, "nums between literals");
  }
  if (fails) {
    std::printf("%d failures\n", fails);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
