// mf_mtx2egr.cpp -- .mtx edge list to MISFIT's binary .egr CSR (offline tool).
//
// Usage: mtx2egr <input.mtx> <output.egr> [--int32]
//
// Replaces tools/efficient_converter.py of anonymous-artifacts/MISFIT (:9-113)
// for inputs of any size: two streaming passes over the text, the entry
// list held in host memory, one sequential write.  Its output for a valid
// input is byte for byte the reference converter's:
//   * the first line that does not start with '%' is the size line; the
//     vertex count is the larger of its first two numbers (:14-22);
//   * every later line with at least two fields is an entry "u v", 1-based;
//     entries with u > vertex count are dropped (:47-52, :97-104);
//   * rows keep the file order of their entries -- no sort, no
//     symmetrisation, no de-duplication;
//   * the int64-sentinel layout: int32 nodes, int32 -1, int64 entries,
//     int64 nindex[n+1], int32 nlist[entries] (:73-78).
// --int32 writes the int32 layout instead (int32 nodes, int32 entries, int32
// nindex[n+1], int32 nlist), which the reference converter cannot produce;
// it is refused beyond 2^31-1 entries.
//
// Differences, for inputs the reference does not handle: a comment line
// after the size line, a field that is not a decimal integer, u < 1, or v
// outside [1, vertex count] is reported as an error (exit code 1) where the
// reference raises or writes an invalid file.
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Line reader over large fread blocks (the inputs run to tens of GB).
struct Reader {
  FILE* f = nullptr;
  std::vector<char> buf;
  size_t pos = 0, len = 0;
  std::string line;
  explicit Reader(const char* path) : f(std::fopen(path, "rb")), buf(1 << 22) {}
  ~Reader() {
    if (f) std::fclose(f);
  }
  bool next() {
    line.clear();
    bool any = false;
    for (;;) {
      if (pos == len) {
        len = std::fread(buf.data(), 1, buf.size(), f);
        pos = 0;
        if (len == 0) return any;
      }
      const char* b = buf.data() + pos;
      const void* nl = std::memchr(b, '\n', len - pos);
      const size_t take = nl ? (size_t)((const char*)nl - b) : len - pos;
      line.append(b, take);
      any = true;
      pos += take;
      if (nl) {
        ++pos;
        return true;
      }
    }
  }
};

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Splits on white space (Python's str.split()).
void fields(const std::string& s, std::vector<std::string>& out) {
  out.clear();
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && is_space(s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !is_space(s[j])) ++j;
    if (j > i) out.emplace_back(s, i, j - i);
    i = j;
  }
}

// A decimal integer with an optional sign (what int() accepts for these files).
bool to_i64(const std::string& t, int64_t* v) {
  size_t i = 0;
  bool neg = false;
  if (i < t.size() && (t[i] == '+' || t[i] == '-')) neg = t[i++] == '-';
  if (i == t.size()) return false;
  int64_t x = 0;
  for (; i < t.size(); ++i) {
    if (t[i] < '0' || t[i] > '9') return false;
    if (x > (INT64_MAX - 9) / 10) return false;
    x = x * 10 + (t[i] - '0');
  }
  *v = neg ? -x : x;
  return true;
}

int fail(const std::string& msg) {
  std::fprintf(stderr, "mtx2egr: %s\n", msg.c_str());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3 || argc > 4 || (argc == 4 && std::strcmp(argv[3], "--int32") != 0))
    return fail("usage: mtx2egr <input.mtx> <output.egr> [--int32]");
  const bool narrow = argc == 4;
  int64_t n = -1;
  std::vector<int64_t> deg;
  std::vector<std::string> fs;
  // pass 1: size line, degrees
  {
    Reader r(argv[1]);
    if (!r.f) return fail(std::string("cannot open ") + argv[1]);
    int64_t lineno = 0;
    while (r.next()) {
      ++lineno;
      if (n < 0) {
        if (!r.line.empty() && r.line[0] == '%') continue;
        fields(r.line, fs);
        int64_t a = 0, b = 0;
        if (fs.size() < 2 || !to_i64(fs[0], &a) || !to_i64(fs[1], &b))
          return fail("line " + std::to_string(lineno) + ": bad size line");
        n = a > b ? a : b;
        if (n < 0 || n > INT32_MAX) return fail("vertex count out of range");
        deg.assign((size_t)n + 1, 0);
        continue;
      }
      fields(r.line, fs);
      if (fs.size() < 2) continue;
      int64_t u = 0, v = 0;
      if (!to_i64(fs[0], &u) || !to_i64(fs[1], &v))
        return fail("line " + std::to_string(lineno) + ": not an entry \"u v\"");
      if (u < 1) return fail("line " + std::to_string(lineno) + ": vertex id below 1");
      if (u > n) continue;
      if (v < 1 || v > n) return fail("line " + std::to_string(lineno) + ": vertex id out of range");
      ++deg[(size_t)u - 1];
    }
    if (n < 0) return fail("no size line");
  }
  std::vector<int64_t> nindex((size_t)n + 1, 0);
  for (int64_t x = 0; x < n; ++x) nindex[(size_t)x + 1] = nindex[(size_t)x] + deg[(size_t)x];
  const int64_t entries = nindex[(size_t)n];
  if (narrow && entries > INT32_MAX) return fail("--int32 cannot hold more than 2^31-1 entries");
  std::vector<int32_t> nlist((size_t)entries);
  // pass 2: rows in file order
  {
    std::vector<int64_t> pos(nindex.begin(), nindex.end() - 1);
    Reader r(argv[1]);
    if (!r.f) return fail(std::string("cannot open ") + argv[1]);
    bool header = true;
    while (r.next()) {
      if (header) {
        if (!r.line.empty() && r.line[0] == '%') continue;
        header = false;
        continue;
      }
      fields(r.line, fs);
      if (fs.size() < 2) continue;
      int64_t u = 0, v = 0;
      to_i64(fs[0], &u);
      to_i64(fs[1], &v);
      if (u > n) continue;
      nlist[(size_t)pos[(size_t)u - 1]++] = (int32_t)(v - 1);
    }
  }
  const std::string tmp = std::string(argv[2]) + ".tmp";
  FILE* out = std::fopen(tmp.c_str(), "wb");
  if (!out) return fail(std::string("cannot write ") + tmp);
  bool ok = true;
  const int32_t n32 = (int32_t)n;
  ok = ok && std::fwrite(&n32, 4, 1, out) == 1;
  if (narrow) {
    const int32_t e32 = (int32_t)entries;
    ok = ok && std::fwrite(&e32, 4, 1, out) == 1;
    std::vector<int32_t> idx(nindex.begin(), nindex.end());
    ok = ok && std::fwrite(idx.data(), 4, idx.size(), out) == idx.size();
  } else {
    const int32_t sentinel = -1;
    ok = ok && std::fwrite(&sentinel, 4, 1, out) == 1;
    ok = ok && std::fwrite(&entries, 8, 1, out) == 1;
    ok = ok && std::fwrite(nindex.data(), 8, nindex.size(), out) == nindex.size();
  }
  ok = ok && std::fwrite(nlist.data(), 4, nlist.size(), out) == nlist.size();
  ok = std::fclose(out) == 0 && ok;
  if (!ok || std::rename(tmp.c_str(), argv[2]) != 0) {
    std::remove(tmp.c_str());
    return fail(std::string("write failed: ") + std::strerror(errno));
  }
  std::printf("%s: %lld vertices, %lld entries, %s layout\n", argv[2], (long long)n, (long long)entries,
              narrow ? "int32" : "int64");
  return 0;
}
