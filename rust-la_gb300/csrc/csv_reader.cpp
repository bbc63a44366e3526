// util::read_csv (src/util.rs:9-35) for Matrix<f64>, with the parser the crate's
// users pass for f64 (`|s| s.parse::<f64>().unwrap()`), as a native reader.
//
// The reference reads the file line by line (BufRead::lines: a line ends at
// '\n', and a '\r' right before it is dropped; invalid UTF-8 panics), splits
// each line at ',' (:18), trims every item (str::trim, Unicode White_Space)
// and parses it; every line must give the first line's item count (:25-27) and
// the file must have a line (:32). Every panic of the reference is LA_BADSHAPE
// here.
//
// f64 parsing follows the grammar of Rust's f64::from_str (std 1.55 and later):
// after lowercasing, Sign? ('inf' | 'infinity' | 'nan' | Number) with
// Number ::= (Digit+ | Digit+ '.' Digit* | Digit* '.' Digit+) ('e' Sign? Digit+)?
// and the value rounded to nearest, ties to even; strtod in the C locale gives
// that rounding once the syntax has been checked here.
//
// The file is read whole, checked for UTF-8 once, cut into lines, and the
// lines are parsed by all host threads straight into the result (the item
// count of every line is known from its commas before any parse).
#include <clocale>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <locale.h>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "la_gpu.h"

namespace {

// Strict UTF-8 (no overlong forms, no surrogates, at most U+10FFFF), as
// String::from_utf8 checks it.
bool valid_utf8(const unsigned char* s, size_t n) {
  size_t i = 0;
  while (i < n) {
    // ASCII runs eight bytes at a time
    while (i + 8 <= n) {
      uint64_t w;
      std::memcpy(&w, s + i, 8);
      if (w & 0x8080808080808080ull) break;
      i += 8;
    }
    if (i >= n) break;
    const unsigned c = s[i];
    if (c < 0x80) { i++; continue; }
    size_t len;
    unsigned cp;
    if (c >= 0xC2 && c <= 0xDF) { len = 2; cp = c & 0x1F; }
    else if (c >= 0xE0 && c <= 0xEF) { len = 3; cp = c & 0x0F; }
    else if (c >= 0xF0 && c <= 0xF4) { len = 4; cp = c & 0x07; }
    else return false;
    if (i + len > n) return false;
    for (size_t k = 1; k < len; k++) {
      const unsigned t = s[i + k];
      if ((t & 0xC0) != 0x80) return false;
      cp = (cp << 6) | (t & 0x3F);
    }
    if ((len == 3 && (cp < 0x800 || (cp >= 0xD800 && cp <= 0xDFFF))) ||
        (len == 4 && (cp < 0x10000 || cp > 0x10FFFF)))
      return false;
    i += len;
  }
  return true;
}

bool white_space(unsigned cp) {
  return (cp >= 0x09 && cp <= 0x0D) || cp == 0x20 || cp == 0x85 || cp == 0xA0 || cp == 0x1680 ||
         (cp >= 0x2000 && cp <= 0x200A) || cp == 0x2028 || cp == 0x2029 || cp == 0x202F ||
         cp == 0x205F || cp == 0x3000;
}

// Length in bytes of the code point starting at s[0] (valid UTF-8).
size_t cp_len(unsigned char c) { return c < 0x80 ? 1 : c < 0xE0 ? 2 : c < 0xF0 ? 3 : 4; }

unsigned decode(const unsigned char* s, size_t len) {
  if (len == 1) return s[0];
  unsigned cp = s[0] & (len == 2 ? 0x1F : len == 3 ? 0x0F : 0x07);
  for (size_t k = 1; k < len; k++) cp = (cp << 6) | (s[k] & 0x3F);
  return cp;
}

// str::trim on [b, e): advance b and retreat e over White_Space code points.
void trim(const unsigned char*& b, const unsigned char*& e) {
  while (b < e) {
    const size_t len = cp_len(*b);
    if (!white_space(decode(b, len))) break;
    b += len;
  }
  while (e > b) {
    const unsigned char* p = e - 1;
    while (p > b && (*p & 0xC0) == 0x80) p--;  // start of the last code point
    if (!white_space(decode(p, (size_t)(e - p)))) break;
    e = p;
  }
}

bool lower_equals(const unsigned char* s, size_t n, const char* word) {
  const size_t w = std::strlen(word);
  if (n != w) return false;
  for (size_t i = 0; i < n; i++) {
    unsigned char c = s[i];
    if (c >= 'A' && c <= 'Z') c = (unsigned char)(c - 'A' + 'a');
    if (c != (unsigned char)word[i]) return false;
  }
  return true;
}

bool is_digit(unsigned char c) { return c >= '0' && c <= '9'; }

// f64::from_str on [s, s + n); false where it returns Err (the reference's
// unwrap then panics).
bool parse_f64(const unsigned char* s, size_t n, locale_t loc, double* out) {
  if (n == 0) return false;
  size_t i = 0;
  bool neg = false;
  if (s[0] == '+' || s[0] == '-') {
    neg = s[0] == '-';
    i = 1;
  }
  const unsigned char* r = s + i;
  const size_t m = n - i;
  if (lower_equals(r, m, "inf") || lower_equals(r, m, "infinity")) {
    *out = neg ? -HUGE_VAL : HUGE_VAL;
    return true;
  }
  if (lower_equals(r, m, "nan")) {
    *out = std::copysign(std::nan(""), neg ? -1.0 : 1.0);
    return true;
  }
  size_t k = 0, d1 = 0, d2 = 0;
  while (k < m && is_digit(r[k])) { k++; d1++; }
  if (k < m && r[k] == '.') {
    k++;
    while (k < m && is_digit(r[k])) { k++; d2++; }
  }
  if (d1 + d2 == 0) return false;
  if (k < m && (r[k] == 'e' || r[k] == 'E')) {
    k++;
    if (k < m && (r[k] == '+' || r[k] == '-')) k++;
    size_t de = 0;
    while (k < m && is_digit(r[k])) { k++; de++; }
    if (de == 0) return false;
  }
  if (k != m) return false;
  // strtod needs a terminated string; the syntax above is a subset of its own
  char small[256];
  std::string big;
  const char* z;
  if (n < sizeof(small)) {
    std::memcpy(small, s, n);
    small[n] = '\0';
    z = small;
  } else {
    big.assign(reinterpret_cast<const char*>(s), n);
    z = big.c_str();
  }
  char* end = nullptr;
  const double v = strtod_l(z, &end, loc);
  if (end != z + n) return false;
  *out = v;
  return true;
}

struct Line {
  size_t b, e;  // byte range without the '\n'
};

}  // namespace

extern "C" la_status la_read_csv_f64(const char* path, double** data, size_t* rows,
                                     size_t* cols) {
  if (!path || !data || !rows || !cols) return LA_INVALID;
  *data = nullptr;
  *rows = 0;
  *cols = 0;
  FILE* f = std::fopen(path, "rb");
  if (!f) return LA_BADSHAPE;  // File::open(..).unwrap() (util.rs:15)
  std::vector<unsigned char> buf;
  {
    // one read of the whole file where its size is known, then whatever follows
    long size = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
    if (std::fseek(f, 0, SEEK_SET) != 0) size = -1;
    if (size > 0) {
      buf.resize((size_t)size);
      buf.resize(std::fread(buf.data(), 1, (size_t)size, f));
    }
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return LA_BADSHAPE;
  }
  const unsigned char* s = buf.data();
  const size_t n = buf.size();
  if (!valid_utf8(s, n)) return LA_BADSHAPE;  // lines() yields Err, unwrap (:17)

  // BufRead::lines: split at '\n'; no empty line after a final '\n'; a '\r'
  // before the '\n' is dropped (trim would remove it from the item anyway).
  std::vector<Line> lines;
  size_t b = 0;
  while (b < n) {
    const void* nl = std::memchr(s + b, '\n', n - b);
    size_t e = nl ? (size_t)(static_cast<const unsigned char*>(nl) - s) : n;
    size_t ee = e;
    if (nl && ee > b && s[ee - 1] == '\r') ee--;
    lines.push_back({b, ee});
    b = nl ? e + 1 : n;
  }
  if (lines.empty()) return LA_BADSHAPE;  // assert!(col_count != None) (:32)

  const size_t R = lines.size();
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  nt = (unsigned)std::min<size_t>(nt, (R + 255) / 256);
  if (nt == 0) nt = 1;

  // item counts (commas + 1) must all equal the first line's (:25-27)
  auto count_items = [&](const Line& l) {
    size_t c = 1;
    for (size_t i = l.b; i < l.e; i++) c += s[i] == ',';
    return c;
  };
  const size_t C = count_items(lines[0]);
  std::atomic<bool> ragged(false);
  {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
      th.emplace_back([&, t]() {
        for (size_t r = t; r < R && !ragged.load(std::memory_order_relaxed); r += nt)
          if (count_items(lines[r]) != C) ragged.store(true);
      });
    for (auto& x : th) x.join();
  }
  if (ragged.load()) return LA_BADSHAPE;

  double* out = static_cast<double*>(std::malloc(R * C * sizeof(double)));
  if (!out) return LA_NOMEM;
  locale_t loc = newlocale(LC_NUMERIC_MASK, "C", (locale_t)0);
  if (loc == (locale_t)0) {
    std::free(out);
    return LA_NOMEM;
  }
  std::atomic<bool> bad(false);
  {
    std::vector<std::thread> th;
    const size_t per = (R + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++)
      th.emplace_back([&, t]() {
        const size_t r0 = t * per, r1 = std::min(R, r0 + per);
        for (size_t r = r0; r < r1 && !bad.load(std::memory_order_relaxed); r++) {
          const Line l = lines[r];
          size_t ib = l.b;
          for (size_t c = 0; c < C; c++) {
            size_t ie = ib;
            while (ie < l.e && s[ie] != ',') ie++;
            const unsigned char* p = s + ib;
            const unsigned char* q = s + ie;
            trim(p, q);
            double v;
            if (!parse_f64(p, (size_t)(q - p), loc, &v)) {
              bad.store(true);
              return;
            }
            out[r * C + c] = v;
            ib = ie + 1;
          }
        }
      });
    for (auto& x : th) x.join();
  }
  freelocale(loc);
  if (bad.load()) {
    std::free(out);
    return LA_BADSHAPE;  // parser(item) is s.parse::<f64>().unwrap()
  }
  *data = out;
  *rows = R;
  *cols = C;
  return LA_OK;
}

extern "C" void la_host_free(void* p) { std::free(p); }
