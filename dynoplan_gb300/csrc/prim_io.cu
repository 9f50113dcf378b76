// prim_io.cu -- motion-primitive files and loader semantics (host code of
// the C ABI in include/dpg_prim_io.h).
//
// The file format is the reference's Trajectories msgpack document
// (Trajectories::load_file_msgpack, called from load_motion_primitives_new,
// src/ompl/robots.cpp:3061-3174):
//   {"data": [{"states": [[x0...], ...], "actions": [[u0...], ...], ...}, ...]}
// Numbers may be float32, float64 or integers; other keys of a motion are
// skipped.  A motion needs at least one state and states - 1 actions.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dpg_prim_io.h"

namespace {

struct Reader {
  const uint8_t *p, *end;
  bool ok = true;

  bool need(size_t n) {
    if ((size_t)(end - p) < n) ok = false;
    return ok;
  }
  uint64_t be(int n) {
    uint64_t v = 0;
    if (!need(n)) return 0;
    for (int i = 0; i < n; i++) v = (v << 8) | p[i];
    p += n;
    return v;
  }
  // container headers: element count, or -1 when the next value is not one
  int64_t map_len() {
    if (!need(1)) return -1;
    const uint8_t t = *p;
    if ((t & 0xf0) == 0x80) { p++; return t & 0x0f; }
    if (t == 0xde) { p++; return (int64_t)be(2); }
    if (t == 0xdf) { p++; return (int64_t)be(4); }
    return -1;
  }
  int64_t array_len() {
    if (!need(1)) return -1;
    const uint8_t t = *p;
    if ((t & 0xf0) == 0x90) { p++; return t & 0x0f; }
    if (t == 0xdc) { p++; return (int64_t)be(2); }
    if (t == 0xdd) { p++; return (int64_t)be(4); }
    return -1;
  }
  bool str(std::string &s) {
    if (!need(1)) return false;
    const uint8_t t = *p;
    size_t n;
    if ((t & 0xe0) == 0xa0) { p++; n = t & 0x1f; }
    else if (t == 0xd9) { p++; n = (size_t)be(1); }
    else if (t == 0xda) { p++; n = (size_t)be(2); }
    else if (t == 0xdb) { p++; n = (size_t)be(4); }
    else return false;
    if (!need(n)) return false;
    s.assign(reinterpret_cast<const char *>(p), n);
    p += n;
    return true;
  }
  bool number(double &v) {
    if (!need(1)) return false;
    const uint8_t t = *p;
    if (t <= 0x7f) { p++; v = t; return true; }
    if (t >= 0xe0) { p++; v = (int8_t)t; return true; }
    p++;
    switch (t) {
      case 0xca: { const uint32_t b = (uint32_t)be(4); float f; std::memcpy(&f, &b, 4); v = f; return ok; }
      case 0xcb: { const uint64_t b = be(8); std::memcpy(&v, &b, 8); return ok; }
      case 0xcc: v = (double)be(1); return ok;
      case 0xcd: v = (double)be(2); return ok;
      case 0xce: v = (double)be(4); return ok;
      case 0xcf: v = (double)be(8); return ok;
      case 0xd0: v = (int8_t)be(1); return ok;
      case 0xd1: v = (int16_t)be(2); return ok;
      case 0xd2: v = (int32_t)be(4); return ok;
      case 0xd3: v = (double)(int64_t)be(8); return ok;
    }
    p--;
    return false;
  }
  // skip one value of any type
  bool skip(int depth = 0) {
    if (depth > 64 || !need(1)) return ok = false;
    const uint8_t t = *p;
    double d;
    std::string s;
    if (number(d) || str(s)) return true;
    int64_t n;
    if ((n = array_len()) >= 0) {
      for (int64_t i = 0; i < n && ok; i++) skip(depth + 1);
      return ok;
    }
    if ((n = map_len()) >= 0) {
      for (int64_t i = 0; i < 2 * n && ok; i++) skip(depth + 1);
      return ok;
    }
    p++;
    switch (t) {
      case 0xc0: case 0xc2: case 0xc3: return true;                         // nil, false, true
      case 0xc4: return need(be(1)) && (p += p[-1], true);                   // bin8
      case 0xc5: { const size_t m = (size_t)be(2); return need(m) && (p += m, true); }
      case 0xc6: { const size_t m = (size_t)be(4); return need(m) && (p += m, true); }
      case 0xd4: return need(2) && (p += 2, true);                           // fixext
      case 0xd5: return need(3) && (p += 3, true);
      case 0xd6: return need(5) && (p += 5, true);
      case 0xd7: return need(9) && (p += 9, true);
      case 0xd8: return need(17) && (p += 17, true);
      case 0xc7: { const size_t m = (size_t)be(1); return need(m + 1) && (p += m + 1, true); }
      case 0xc8: { const size_t m = (size_t)be(2); return need(m + 1) && (p += m + 1, true); }
      case 0xc9: { const size_t m = (size_t)be(4); return need(m + 1) && (p += m + 1, true); }
    }
    return ok = false;
  }
  // array of rows of numbers; every row has the same width (set on the first)
  bool rows(std::vector<double> &out, int64_t &n_rows, int32_t &width) {
    const int64_t n = array_len();
    if (n < 0) return false;
    n_rows = n;
    for (int64_t r = 0; r < n; r++) {
      const int64_t w = array_len();
      if (w < 0 || (width >= 0 && w != width)) return false;
      width = (int32_t)w;
      for (int64_t j = 0; j < w; j++) {
        double v;
        if (!number(v)) return false;
        out.push_back(v);
      }
    }
    return ok;
  }
};

struct Motions {
  std::vector<int32_t> len;
  std::vector<double> states, actions;
  int32_t nx = -1, nu = -1;
};

int parse(const char *path, int32_t max_motions, Motions &m) {
  if (!path) return DPG_ERR_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return DPG_ERR_ARG;
  std::vector<uint8_t> buf;
  uint8_t tmp[1 << 16];
  size_t got;
  while ((got = std::fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + got);
  std::fclose(f);
  Reader r{buf.data(), buf.data() + buf.size()};
  const int64_t top = r.map_len();
  if (top < 0) return DPG_ERR_ARG;
  bool have_data = false;
  for (int64_t i = 0; i < top; i++) {
    std::string key;
    if (!r.str(key)) return DPG_ERR_ARG;
    if (key != "data") {
      if (!r.skip()) return DPG_ERR_ARG;
      continue;
    }
    have_data = true;
    const int64_t n = r.array_len();
    if (n < 0) return DPG_ERR_ARG;
    for (int64_t t = 0; t < n; t++) {
      const bool keep = max_motions <= 0 || (int64_t)m.len.size() < max_motions;
      const int64_t fields = r.map_len();
      if (fields < 0) return DPG_ERR_ARG;
      std::vector<double> st, ac;
      int64_t ns = -1, na = -1;
      for (int64_t k = 0; k < fields; k++) {
        std::string fk;
        if (!r.str(fk)) return DPG_ERR_ARG;
        if (keep && fk == "states") {
          if (!r.rows(st, ns, m.nx)) return DPG_ERR_ARG;
        } else if (keep && fk == "actions") {
          if (!r.rows(ac, na, m.nu)) return DPG_ERR_ARG;
        } else if (!r.skip()) {
          return DPG_ERR_ARG;
        }
      }
      if (!keep) continue;
      if (ns < 1 || na != ns - 1 || ns > 32767) return DPG_ERR_ARG;
      m.len.push_back((int32_t)ns);
      m.states.insert(m.states.end(), st.begin(), st.end());
      m.actions.insert(m.actions.end(), ac.begin(), ac.end());
    }
  }
  if (!have_data || !r.ok) return DPG_ERR_ARG;
  if (m.nu < 0) m.nu = 0;  // motions of one state only
  return DPG_OK;
}

// ---- writer ----------------------------------------------------------------
struct Writer {
  std::vector<uint8_t> b;
  void be(uint64_t v, int n) {
    for (int i = n - 1; i >= 0; i--) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void map(uint32_t n) {
    if (n < 16) b.push_back((uint8_t)(0x80 | n));
    else if (n < 65536) { b.push_back(0xde); be(n, 2); }
    else { b.push_back(0xdf); be(n, 4); }
  }
  void array(uint64_t n) {
    if (n < 16) b.push_back((uint8_t)(0x90 | n));
    else if (n < 65536) { b.push_back(0xdc); be(n, 2); }
    else { b.push_back(0xdd); be(n, 4); }
  }
  void str(const char *s) {
    const size_t n = std::strlen(s);
    b.push_back((uint8_t)(0xa0 | n));  // keys here are short
    b.insert(b.end(), s, s + n);
  }
  // compact: float32 when the value is exactly a float32 (how the bundled
  // files encode 0.0, 0.5, ...), else float64; lossless either way
  void num(double v, bool compact) {
    if (compact && (double)(float)v == v) {
      const float f = (float)v;
      uint32_t u;
      std::memcpy(&u, &f, 4);
      b.push_back(0xca);
      be(u, 4);
    } else {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      b.push_back(0xcb);
      be(u, 8);
    }
  }
  void rows(const double *x, int64_t n, int32_t w, bool compact) {
    array((uint64_t)n);
    for (int64_t r = 0; r < n; r++) {
      array((uint64_t)w);
      for (int32_t j = 0; j < w; j++) num(x[r * w + j], compact);
    }
  }
};

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int dpg_primitives_file_info(const char *path, int32_t max_motions, int32_t *P, int64_t *S, int64_t *A,
                             int32_t *nx, int32_t *nu) {
  Motions m;
  const int rc = parse(path, max_motions, m);
  if (rc) return rc;
  int64_t s = 0, a = 0;
  for (int32_t l : m.len) { s += l; a += l - 1; }
  if (P) *P = (int32_t)m.len.size();
  if (S) *S = s;
  if (A) *A = a;
  if (nx) *nx = m.nx;
  if (nu) *nu = m.nu;
  return DPG_OK;
}

int dpg_primitives_file_read(const char *path, int32_t max_motions, int32_t *len, double *states,
                             double *actions) {
  if (!len || !states) return DPG_ERR_ARG;
  Motions m;
  const int rc = parse(path, max_motions, m);
  if (rc) return rc;
  std::memcpy(len, m.len.data(), sizeof(int32_t) * m.len.size());
  std::memcpy(states, m.states.data(), sizeof(double) * m.states.size());
  if (!m.actions.empty()) {
    if (!actions) return DPG_ERR_ARG;
    std::memcpy(actions, m.actions.data(), sizeof(double) * m.actions.size());
  }
  return DPG_OK;
}

int dpg_primitives_file_write(const char *path, int32_t P, const int32_t *len, const double *states,
                              const double *actions, int32_t nx, int32_t nu, int32_t compact) {
  if (!path || P < 0 || (P > 0 && (!len || !states)) || nx <= 0 || nu < 0) return DPG_ERR_ARG;
  Writer w;
  w.map(1);
  w.str("data");
  w.array((uint64_t)P);
  int64_t s = 0, a = 0;
  for (int32_t p = 0; p < P; p++) {
    if (len[p] < 1) return DPG_ERR_ARG;
    if (len[p] > 1 && (!actions || nu <= 0)) return DPG_ERR_ARG;
    w.map(2);
    w.str("actions");
    w.rows(actions ? actions + a * nu : nullptr, len[p] - 1, nu, compact != 0);
    w.str("states");
    w.rows(states + s * nx, len[p], nx, compact != 0);
    s += len[p];
    a += len[p] - 1;
  }
  FILE *f = std::fopen(path, "wb");
  if (!f) return DPG_ERR_ARG;
  const bool ok = std::fwrite(w.b.data(), 1, w.b.size(), f) == w.b.size();
  return (std::fclose(f) == 0 && ok) ? DPG_OK : DPG_ERR_ARG;
}

int dpg_primitives_prepare(int32_t kind, int32_t P, const int32_t *len, double *states, int32_t nx, double noise,
                           uint64_t seed) {
  if (P < 0 || (P > 0 && (!len || !states)) || nx <= 0 || !(noise >= 0)) return DPG_ERR_ARG;
  uint64_t s = seed;
  auto uni = [&] {  // uniform in [-1, 1)
    return (double)(splitmix(s) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  };
  int64_t off = 0;
  for (int32_t p = 0; p < P; p++) {
    if (len[p] < 1) return DPG_ERR_ARG;
    double *first = states + off * nx, *last = states + (off + len[p] - 1) * nx;
    for (int32_t j = 0; j < nx; j++) first[j] += noise * uni();
    for (int32_t j = 0; j < nx; j++) last[j] += noise * uni();
    if (kind == DPG_ROBOT_QUAD3D && nx >= 7)
      for (int32_t k = 0; k < len[p]; k++) {
        double *q = states + (off + k) * nx + 3;
        const double n = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        if (n > 0)
          for (int i = 0; i < 4; i++) q[i] /= n;
      }
    off += len[p];
  }
  return DPG_OK;
}

}  // extern "C"
