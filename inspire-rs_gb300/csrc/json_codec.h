// json_codec.h -- the JSON reader and writer of the wire codecs (host code
// only, plain C++17, no CUDA): a strict reader for the shapes serde_json
// writes (objects, arrays, unsigned integers, booleans, strings, null) and an
// append-only writer of serde_json's compact form.
//
// Numbers follow serde_json's grammar for unsigned integers: one or more
// digits, no sign, no fraction or exponent, and no leading zero ("0" is a
// number, "07" is not).  Compact integer arrays ("1,22,333") take a SWAR fast
// path; every other form goes through the checked path, which reports the
// error.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace igjson {

// ---------------------------------------------------------------- parser
struct Json {
  const char* p;
  const char* end;
  std::string err;

  bool fail(const std::string& m) {
    if (err.empty()) err = m + " at byte " + std::to_string(pos());
    return false;
  }
  size_t pos() const { return (size_t)(p - begin); }
  const char* begin;

  void ws() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) p++;
  }
  bool eat(char c) {
    ws();
    if (p < end && *p == c) {
      p++;
      return true;
    }
    return false;
  }
  bool expect(char c) { return eat(c) || fail(std::string("expected '") + c + "'"); }
  bool str(std::string& out) {
    ws();
    if (p >= end || *p != '"') return fail("expected a string");
    p++;
    out.clear();
    while (p < end && *p != '"') {
      if (*p == '\\') {
        if (p + 1 >= end) return fail("bad escape");
        p++;
        const char c = *p;
        out.push_back(c == 'n' ? '\n' : c == 't' ? '\t' : c == 'r' ? '\r' : c);  // keys here are plain ASCII
        p++;
        continue;
      }
      out.push_back(*p++);
    }
    if (p >= end) return fail("unterminated string");
    p++;
    return true;
  }
  bool u64(uint64_t& v) {
    ws();
    const char* q = p;
    uint64_t x = 0;
    // up to 19 digits cannot overflow; a 20th is checked
    int n = 0;
    while (q < end && (unsigned)(*q - '0') < 10u && n < 19) {
      x = x * 10 + (uint64_t)(*q - '0');
      q++;
      n++;
    }
    if (n == 0) return fail("expected an unsigned integer");
    if (*p == '0' && n > 1) return fail("invalid number (leading zero)");
    if (q < end && (unsigned)(*q - '0') < 10u) {
      const uint64_t d = (uint64_t)(*q - '0');
      if (x > (UINT64_MAX - d) / 10) return fail("integer overflow");
      x = x * 10 + d;
      q++;
      if (q < end && (unsigned)(*q - '0') < 10u) return fail("integer overflow");
    }
    p = q;
    if (p < end && (*p == '.' || *p == 'e' || *p == 'E')) return fail("expected an integer");
    v = x;
    return true;
  }
  // array of at most cap u64 into out; *n receives the count
  bool u64_array_into(uint64_t* out, size_t cap, size_t* n) {
    *n = 0;
    if (!expect('[')) return false;
    if (eat(']')) return true;
    if (compact_run(out, cap, n)) return expect(']');
    for (;;) {
      uint64_t v;
      // compact runs ("123,45,...") eight bytes at a time; anything else
      // (whitespace, long or malformed numbers, the last bytes) takes u64()
      if (!digits_fast(v) && !u64(v)) return false;
      if (*n >= cap) return fail("array too long");
      out[(*n)++] = v;
      if (p < end && *p == ',') {
        p++;
        continue;
      }
      if (!eat(',')) break;
    }
    return expect(']');
  }
  // One number of 1..16 digits directly followed by ',' or ']', with 17
  // readable bytes: parsed by SWAR on little-endian 8-byte words (x86-64 and
  // AArch64 alike).  Returns false, consuming nothing, for every other case.
  bool digits_fast(uint64_t& v) {
    if (end - p < 17) return false;
    uint64_t w0, w1;
    memcpy(&w0, p, 8);
    memcpy(&w1, p + 8, 8);
    const int n0 = digit_run(w0);
    if (n0 == 0) return false;
    uint64_t x = swar_value(w0, n0);
    int len = n0;
    if (n0 == 8) {
      const int n1 = digit_run(w1);
      if (n1 == 8) return false;  // 17+ digits: the checked path
      if (n1) x = x * pow10(n1) + swar_value(w1, n1);
      len += n1;
    }
    const char t = p[len];
    if (t != ',' && t != ']') return false;
    if (len > 1 && *p == '0') return false;  // leading zero: the checked path reports it
    p += len;
    v = x;
    return true;
  }
  // A compact run "d,d,...,d" of unsigned integers of 1..16 digits up to
  // the closing ']': the commas are located first, eight bytes at a time,
  // then every number is parsed on its own (SWAR), so that parsing one
  // number does not wait for the end of the previous one to be found.
  // Returns false, consuming nothing, for any other array body (whitespace,
  // signs, empty or long elements, too many elements): the checked path
  // then parses it and reports its errors.
  bool compact_run(uint64_t* out, size_t cap, size_t* n) {
    const char* s = p;
    const char* q = s;
    cpos.clear();
    constexpr uint64_t H = 0x8080808080808080ull;
    bool stop = false;
    while (!stop && end - q >= 8) {
      uint64_t w;
      memcpy(&w, q, 8);
      const uint64_t comma = byte_eq(w, ',');
      const uint64_t other = ~(digit_bits(w) | comma) & H;
      uint64_t cm = comma;
      if (other) {
        cm &= (other & (0 - other)) - 1;  // the commas before the first other byte
        stop = true;
      }
      for (; cm; cm &= cm - 1) cpos.push_back((uint32_t)(q - s) + (uint32_t)(__builtin_ctzll(cm) >> 3));
      q += other ? (__builtin_ctzll(other) >> 3) : 8;
    }
    if (!stop)
      for (; q < end && ((unsigned)(*q - '0') < 10u || *q == ','); q++)
        if (*q == ',') cpos.push_back((uint32_t)(q - s));
    if (q >= end || *q != ']' || q == s) return false;
    const size_t k = cpos.size() + 1;
    if (k > cap) return false;
    uint32_t start = 0;
    for (size_t i = 0; i < k; i++) {
      const uint32_t stop_at = i + 1 < k ? cpos[i] : (uint32_t)(q - s);
      const uint32_t len = stop_at - start;
      if (len == 0 || len > 16) return false;
      const char* a = s + start;
      if (len > 1 && *a == '0') return false;  // leading zero: the checked path reports it
      uint64_t v;
      if (end - a >= 16) {
        // branch-free over the length: 8- and 9-digit values alternate at random
        uint64_t w0, w1;
        memcpy(&w0, a, 8);
        memcpy(&w1, a + 8, 8);
        const int l0 = len < 8 ? (int)len : 8, l1 = (int)len - l0;
        v = swar_any(w0, l0) * kPow10[l1] + swar_any(w1, l1);
      } else {
        v = 0;
        for (uint32_t j = 0; j < len; j++) v = v * 10 + (uint64_t)(a[j] - '0');
      }
      out[i] = v;
      start = stop_at + 1;
    }
    *n = k;
    p = q;
    return true;
  }
  std::vector<uint32_t> cpos;  // comma offsets of the current compact run
  static constexpr uint64_t kPow10[9] = {1, 10, 100, 1000, 10000, 100000, 1000000, 10000000, 100000000};
  // value of the first n (0..8) digits of w; 0 for n = 0
  static uint64_t swar_any(uint64_t w, int n) {
    uint64_t d = w - 0x3030303030303030ull;
    const int sh = 4 * (8 - n);  // two shifts: n = 0 clears d without a 64-bit shift
    d = (d << sh) << sh;
    d = (d * 10 + (d >> 8)) & 0x00ff00ff00ff00ffull;
    d = (d * 100 + (d >> 16)) & 0x0000ffff0000ffffull;
    return (d * 10000 + (d >> 32)) & 0xffffffffull;
  }
  // high bit of every byte of w equal to c
  static uint64_t byte_eq(uint64_t w, char c) {
    const uint64_t L7 = 0x7f7f7f7f7f7f7f7full;
    const uint64_t x = w ^ (0x0101010101010101ull * (uint8_t)c);
    return ~(((x & L7) + L7) | x | L7);
  }
  // high bit of every ASCII digit byte of w
  static uint64_t digit_bits(uint64_t w) {
    const uint64_t H = 0x8080808080808080ull;
    const uint64_t ge0 = ((w | H) - 0x3030303030303030ull) & H;
    const uint64_t ge10 = ((w | H) - 0x3a3a3a3a3a3a3a3aull) & H;
    return ge0 & ~ge10 & ~(w & H);
  }
  // number of leading ASCII digits in the 8 bytes of w (first byte lowest)
  static int digit_run(uint64_t w) {
    const uint64_t H = 0x8080808080808080ull;
    const uint64_t ge0 = ((w | H) - 0x3030303030303030ull) & H;  // (b & 0x7f) >= '0'
    const uint64_t ge10 = ((w | H) - 0x3a3a3a3a3a3a3a3aull) & H; // (b & 0x7f) > '9'
    const uint64_t digit = ge0 & ~ge10 & ~(w & H);
    const uint64_t other = ~digit & H;
    return other ? __builtin_ctzll(other) >> 3 : 8;
  }
  // value of the first n (1..8) digits of w
  static uint64_t swar_value(uint64_t w, int n) {
    uint64_t d = w - 0x3030303030303030ull;  // the low n bytes are 0..9
    d <<= 8 * (8 - n);                        // right-align: leading zero digits
    d = (d * 10 + (d >> 8)) & 0x00ff00ff00ff00ffull;     // digit pairs
    d = (d * 100 + (d >> 16)) & 0x0000ffff0000ffffull;   // groups of four
    return (d * 10000 + (d >> 32)) & 0xffffffffull;      // eight digits
  }
  static uint64_t pow10(int n) {
    uint64_t r = 1;
    while (n--) r *= 10;
    return r;
  }
  bool boolean(bool& b) {
    ws();
    if (end - p >= 4 && memcmp(p, "true", 4) == 0) {
      p += 4;
      b = true;
      return true;
    }
    if (end - p >= 5 && memcmp(p, "false", 5) == 0) {
      p += 5;
      b = false;
      return true;
    }
    return fail("expected a boolean");
  }
  // skip any JSON value (unknown fields)
  bool skip() {
    ws();
    if (p >= end) return fail("unexpected end");
    if (*p == '"') {
      std::string s;
      return str(s);
    }
    if (*p == '{' || *p == '[') {
      const char open = *p, close = open == '{' ? '}' : ']';
      p++;
      if (eat(close)) return true;
      do {
        if (open == '{') {
          std::string k;
          if (!str(k) || !expect(':')) return false;
        }
        if (!skip()) return false;
      } while (eat(','));
      return expect(close);
    }
    if (*p == 't' || *p == 'f') {
      bool b;
      return boolean(b);
    }
    if (end - p >= 4 && memcmp(p, "null", 4) == 0) {
      p += 4;
      return true;
    }
    // number (possibly signed / fractional)
    const char* s = p;
    while (p < end && (*p == '+' || *p == '-' || *p == '.' || *p == 'e' || *p == 'E' || (*p >= '0' && *p <= '9')))
      p++;
    return p > s || fail("unexpected character");
  }
  bool null() {
    ws();
    if (end - p >= 4 && memcmp(p, "null", 4) == 0) {
      p += 4;
      return true;
    }
    return false;
  }
  // object: calls field(key) for each key; field consumes the value
  template <class F>
  bool object(F&& field) {
    if (!expect('{')) return false;
    if (eat('}')) return true;
    do {
      std::string k;
      if (!str(k) || !expect(':')) return false;
      if (!field(k)) return false;
    } while (eat(','));
    return expect('}');
  }
  template <class F>
  bool array(F&& elem) {
    if (!expect('[')) return false;
    if (eat(']')) return true;
    size_t i = 0;
    do {
      if (!elem(i++)) return false;
    } while (eat(','));
    return expect(']');
  }
};

// ---------------------------------------------------------------- writer
struct Out {
  // the output so far: n bytes of buf (uninitialised beyond them, so room
  // reserved ahead of the writes costs no fill)
  std::unique_ptr<char[]> buf;
  size_t cap = 0, n = 0;
  void reserve(size_t c) {
    if (c <= cap) return;
    std::unique_ptr<char[]> b(new char[c]);
    if (n) memcpy(b.get(), buf.get(), n);
    buf = std::move(b);
    cap = c;
  }
  void room(size_t k) {
    if (n + k > cap) reserve(std::max(cap * 2, n + k + 4096));
  }
  const char* data() const { return buf.get(); }
  bool equals(const std::string& w) const { return n == w.size() && (n == 0 || memcmp(buf.get(), w.data(), n) == 0); }
  void ch(char c) {
    room(1);
    buf[n++] = c;
  }
  void lit(const char* x) {
    const size_t k = strlen(x);
    room(k);
    memcpy(&buf[n], x, k);
    n += k;
  }
  // Decimal digits of v (1..20): for v >= 10, t = floor(bits * 1233 / 4096)
  // (1233 / 4096 ~ log10 2) is the digit count or one less, settled by one
  // comparison.
  static int digits(uint64_t v) {
    static constexpr uint64_t p10[20] = {1ull,
                                         10ull,
                                         100ull,
                                         1000ull,
                                         10000ull,
                                         100000ull,
                                         1000000ull,
                                         10000000ull,
                                         100000000ull,
                                         1000000000ull,
                                         10000000000ull,
                                         100000000000ull,
                                         1000000000000ull,
                                         10000000000000ull,
                                         100000000000000ull,
                                         1000000000000000ull,
                                         10000000000000000ull,
                                         100000000000000000ull,
                                         1000000000000000000ull,
                                         10000000000000000000ull};
    if (v < 10) return 1;
    const int t = ((64 - __builtin_clzll(v)) * 1233) >> 12;  // t <= 19
    return t + (v >= p10[t] ? 1 : 0);
  }
  // The eight decimal digits of x < 10^8, zero-padded, as ASCII in a u64
  // whose lowest byte (first in memory on little-endian hosts, x86-64 and
  // AArch64 alike) is the leading digit.  SWAR: x is split into 4 + 4 digits
  // in 32-bit lanes, then 2 + 2 in 16-bit lanes, then 1 + 1 in bytes; each
  // lane's quotient is a multiply and shift, exact in its range
  // (t / 100 = (t * 5243) >> 19 for t < 43699, u / 10 = (u * 103) >> 10 for
  // u < 179), and no lane's product reaches the next lane.
  static uint64_t ascii8(uint32_t x) {
    const uint32_t hi = x / 10000;
    uint64_t v = hi | ((uint64_t)(x - hi * 10000) << 32);
    const uint64_t q = ((v * 5243) >> 19) & 0x0000007F0000007Full;
    v = q | ((v - q * 100) << 16);
    const uint64_t q2 = ((v * 103) >> 10) & 0x000F000F000F000Full;
    v = q2 | ((v - q2 * 10) << 8);
    return v | 0x3030303030303030ull;
  }
  // v in decimal at p; returns the length.  Needs room for 20 bytes: numbers
  // below 10^16 are stored as whole 8-byte words, so up to 8 bytes past the
  // number are written too (the next writes overwrite them, or done() cuts
  // them off).
  static int put_num(char* p, uint64_t v) {
    if (v < 100000000ull) {
      const int len = digits(v);
      const uint64_t w = ascii8((uint32_t)v) >> (8 * (8 - len));
      memcpy(p, &w, 8);
      return len;
    }
    if (v < 10000000000000000ull) {
      const uint64_t hi = v / 100000000ull;
      const int hl = put_num(p, hi);
      const uint64_t w = ascii8((uint32_t)(v - hi * 100000000ull));
      memcpy(p + hl, &w, 8);
      return hl + 8;
    }
    // 17 to 20 digits: two per step from the right
    static constexpr char d2[201] =
        "00010203040506070809101112131415161718192021222324252627282930313233343536373839"
        "40414243444546474849505152535455565758596061626364656667686970717273747576777879"
        "8081828384858687888990919293949596979899";
    const int len = digits(v);
    char* e = p + len;
    while (v >= 100) {
      const uint64_t q = v / 100;
      const unsigned r = (unsigned)(v - q * 100);
      e -= 2;
      memcpy(e, d2 + 2 * r, 2);
      v = q;
    }
    if (v >= 10) {
      e -= 2;
      memcpy(e, d2 + 2 * v, 2);
    } else {
      *--e = (char)('0' + v);
    }
    return len;
  }
  void num(uint64_t v) {
    room(20);
    n += (size_t)put_num(&buf[n], v);
  }
  // "a0,a1,...,ak-1" (no brackets), room reserved once.  Values below 10^9
  // (every residue) take a path without data-dependent branches (8- and
  // 9-digit residues are about equally common, so a branch on the length
  // would be mispredicted): the nine-digit zero-padded string is formed in
  // a 128-bit value, shifted by the length and stored as 16 bytes.
  void nums(const uint64_t* a, size_t k) {
    room(21 * k + 1);
    char* p = &buf[n];
    char* const p0 = p;
    for (size_t i = 0; i < k; i++) {
      if (i) *p++ = ',';
      const uint64_t v = a[i];
      if (v < 1000000000ull) {
        const uint32_t hi = (uint32_t)(v / 100000000ull);
        const uint64_t w = ascii8((uint32_t)(v - (uint64_t)hi * 100000000ull));
        const int len = digits(v);
        const unsigned __int128 z = (((unsigned __int128)w << 8) | (uint64_t)('0' + hi)) >> (8 * (9 - len));
        memcpy(p, &z, 16);
        p += len;
      } else {
        p += put_num(p, v);
      }
    }
    n += (size_t)(p - p0);
  }
  std::string done() const { return std::string(buf.get(), n); }
};

}  // namespace igjson
