// mf_mkbatches.cpp -- batch folders of existing edges sampled from a .egr
// graph (offline tool).
//
// Usage: mkbatches <graph.egr> <out_folder> <batch_size> <num_batches>
//                  [uniform|low_degree|preferential] [seed]
//
// Replaces the reference's three batch generators (anonymous-artifacts/MISFIT
// tools/generate_test_batches.py:32-89, generate_low_degree_batches.py,
// generate_preferential_batches.py) for graphs of any size.  They share one
// recipe, which this tool follows:
//   * draw CSR entries (u, v) of the graph:
//       uniform       -- an entry position uniform over all entries;
//       low_degree    -- u with probability proportional to 1/deg(u) among
//                        vertices with entries, then a uniform entry of its row;
//       preferential  -- u proportional to deg(u), then a uniform entry of its row
//                        (so every entry is equally likely, as in uniform; the
//                        recipes differ only in how repeats and self-loops fall);
//   * skip self-loops, keep each unordered pair once, until batch_size x
//     num_batches distinct pairs are found;
//   * shuffle them, write batch k (1-based) to <out_folder>/k.mtx, one
//     "min max" line per pair, 1-based ids.
// Every line is an existing edge, so every line is a delete when the
// reference flags the batch against the base graph.  The draws come from
// this tool's own generator (xoshiro256** seeded through splitmix64, the
// published algorithms of Blackman and Vigna), so the files follow the same
// distributions as the reference's but are not the same files.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_set>
#include <vector>

#include <sys/stat.h>

namespace {

int fail(const std::string& msg) {
  std::fprintf(stderr, "mkbatches: %s\n", msg.c_str());
  return 1;
}

// splitmix64 (seeding) and xoshiro256** (draws).
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t z = seed;
    for (auto& w : s) {
      z += 0x9e3779b97f4a7c15ull;
      uint64_t x = z;
      x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
      x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
      w = x ^ (x >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform in [0, bound) by rejection (no modulo bias)
  uint64_t below(uint64_t bound) {
    const uint64_t lim = UINT64_MAX - UINT64_MAX % bound;
    uint64_t x;
    do x = next(); while (x >= lim);
    return x % bound;
  }
  double unit() { return (double)(next() >> 11) * 0x1.0p-53; }
};

bool read_egr(const char* path, int32_t* n, std::vector<int64_t>& nindex, std::vector<int32_t>& nlist) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  int32_t nodes = 0, e32 = 0;
  uint64_t entries = 0;
  bool ok = std::fread(&nodes, 4, 1, f) == 1 && std::fread(&e32, 4, 1, f) == 1 && nodes >= 0;
  bool wide = false;
  if (ok && e32 == -1) {
    ok = std::fread(&entries, 8, 1, f) == 1;
    wide = true;
  } else if (ok) {
    ok = e32 >= 0;
    entries = (uint64_t)e32;
  }
  if (ok) {
    nindex.resize((size_t)nodes + 1);
    if (wide) {
      ok = std::fread(nindex.data(), 8, nindex.size(), f) == nindex.size();
    } else {
      std::vector<int32_t> t(nindex.size());
      ok = std::fread(t.data(), 4, t.size(), f) == t.size();
      for (size_t i = 0; ok && i < t.size(); ++i) nindex[i] = t[i];
    }
  }
  if (ok) {
    nlist.resize(entries);
    ok = std::fread(nlist.data(), 4, entries, f) == entries;
  }
  std::fclose(f);
  if (!ok) return false;
  for (int32_t x = 0; x < nodes; ++x)
    if (nindex[(size_t)x] > nindex[(size_t)x + 1]) return false;
  if (nindex[0] != 0 || (uint64_t)nindex[(size_t)nodes] != entries) return false;
  for (int32_t y : nlist)
    if (y < 0 || y >= nodes) return false;
  *n = nodes;
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5 || argc > 7)
    return fail("usage: mkbatches <graph.egr> <out_folder> <batch_size> <num_batches> "
                "[uniform|low_degree|preferential] [seed]");
  const std::string mode = argc > 5 ? argv[5] : "uniform";
  if (mode != "uniform" && mode != "low_degree" && mode != "preferential") return fail("unknown mode " + mode);
  char* end = nullptr;
  const long long bs = std::strtoll(argv[3], &end, 10);
  if (*end || bs <= 0) return fail("batch_size must be a positive integer");
  const long long nb = std::strtoll(argv[4], &end, 10);
  if (*end || nb <= 0) return fail("num_batches must be a positive integer");
  uint64_t seed = 42;
  if (argc > 6) {
    seed = std::strtoull(argv[6], &end, 10);
    if (*end) return fail("seed must be an integer");
  }
  int32_t n = 0;
  std::vector<int64_t> nindex;
  std::vector<int32_t> nlist;
  if (!read_egr(argv[1], &n, nindex, nlist)) return fail(std::string("cannot read a valid .egr from ") + argv[1]);
  const uint64_t entries = nlist.size();
  const uint64_t need = (uint64_t)bs * (uint64_t)nb;
  if (need > entries) return fail("need more pairs than the graph has entries");

  // vertex distribution of the weighted modes (cumulative weights)
  std::vector<double> cdf;
  if (mode != "uniform") {
    cdf.resize((size_t)n);
    double acc = 0.0;
    for (int32_t x = 0; x < n; ++x) {
      const int64_t d = nindex[(size_t)x + 1] - nindex[(size_t)x];
      acc += d > 0 ? (mode == "preferential" ? (double)d : 1.0 / (double)d) : 0.0;
      cdf[(size_t)x] = acc;
    }
    if (acc <= 0.0) return fail("the graph has no entries to sample");
  }
  Rng rng(seed);
  std::unordered_set<uint64_t> seen;
  seen.reserve((size_t)need * 2);
  std::vector<uint64_t> pairs;
  pairs.reserve((size_t)need);
  const uint64_t max_draws = 200 * need + 100000;
  for (uint64_t draw = 0; pairs.size() < need; ++draw) {
    if (draw >= max_draws) return fail("could not find enough distinct non-self-loop pairs");
    int64_t pos;
    int32_t u;
    if (mode == "uniform") {
      pos = (int64_t)rng.below(entries);
      // the row holding entry pos: last x with nindex[x] <= pos
      int64_t lo = 0, hi = n;
      while (hi - lo > 1) {
        const int64_t mid = (lo + hi) / 2;
        if (nindex[(size_t)mid] <= pos) lo = mid; else hi = mid;
      }
      u = (int32_t)lo;
    } else {
      const double t = rng.unit() * cdf.back();
      int64_t lo = 0, hi = n - 1;  // first x with cdf[x] > t
      while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (cdf[(size_t)mid] > t) hi = mid; else lo = mid + 1;
      }
      u = (int32_t)lo;
      const int64_t d = nindex[(size_t)u + 1] - nindex[(size_t)u];
      if (d <= 0) continue;
      pos = nindex[(size_t)u] + (int64_t)rng.below((uint64_t)d);
    }
    const int32_t v = nlist[(size_t)pos];
    if (u == v) continue;
    const uint64_t a = (uint64_t)(u < v ? u : v), b = (uint64_t)(u < v ? v : u);
    const uint64_t key = (a << 32) | b;
    if (seen.insert(key).second) pairs.push_back(key);
  }
  for (size_t i = pairs.size(); i > 1; --i) std::swap(pairs[i - 1], pairs[(size_t)rng.below(i)]);

  if (mkdir(argv[2], 0755) != 0 && errno != EEXIST) return fail(std::string("cannot create ") + argv[2]);
  for (long long k = 1; k <= nb; ++k) {
    const std::string path = std::string(argv[2]) + "/" + std::to_string(k) + ".mtx";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return fail("cannot write " + path);
    bool ok = true;
    for (long long i = (k - 1) * bs; i < k * bs; ++i) {
      const uint64_t key = pairs[(size_t)i];
      ok = ok && std::fprintf(f, "%llu %llu\n", (unsigned long long)(key >> 32) + 1,
                              (unsigned long long)(key & 0xffffffffull) + 1) > 0;
    }
    if (std::fclose(f) != 0 || !ok) return fail("write failed: " + path);
  }
  std::printf("%s: %lld batches of %lld %s-sampled existing edges\n", argv[2], nb, bs, mode.c_str());
  return 0;
}
