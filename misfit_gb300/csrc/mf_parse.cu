// mf_parse.cu -- batch files parsed on the device.
//
// A batch file is text: one update per line, "u v" with 1-based ids
// (core/cli_setup.h:66-82).  The reference reads a line with
// `iss >> src >> dst`: leading white space is skipped, an optional sign and
// decimal digits make a number (one that does not fit an int fails), and
// the line counts only if both numbers parse; anything after the second
// number is ignored.  Ids are then made 0-based, and lines with an id out of
// range or with equal ids are dropped.  Here the file is copied to the
// device once; a scan over the bytes finds the line starts, one thread parses
// each line with those rules, and the valid lines are compacted in file
// order.  The insert/delete flags are computed against the current graph
// (mf_flag_updates), as the reference does for every batch before any runs.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mf_internal.cuh"

namespace mf {
namespace {

constexpr int kTB = 256;

inline unsigned grid_for(int64_t n, int per = kTB) {
  int64_t g = (n + per - 1) / per;
  if (g < 1) g = 1;
  if (g > (1 << 30)) g = 1 << 30;
  return (unsigned)g;
}

__global__ void k_line_starts(const char* text, int64_t size, uint8_t* starts) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < size) starts[i] = (i == 0 || text[i - 1] == '\n') ? 1 : 0;
}

__global__ void k_line_offsets(const uint8_t* starts, const int64_t* pos, int64_t size, int64_t* line_begin) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < size && starts[i]) line_begin[pos[i]] = i;
}

__device__ __forceinline__ bool is_space(char ch) {
  return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f';
}

// One number as `istream >> int` reads it, from text[*k] on (white space
// first); false when there is none or it does not fit an int.
__device__ bool parse_int(const char* text, int64_t end, int64_t* k, int64_t* out) {
  int64_t i = *k;
  while (i < end && is_space(text[i])) ++i;
  bool neg = false;
  if (i < end && (text[i] == '+' || text[i] == '-')) {
    neg = text[i] == '-';
    ++i;
  }
  if (i >= end || text[i] < '0' || text[i] > '9') return false;
  int64_t v = 0;
  while (i < end && text[i] >= '0' && text[i] <= '9') {
    v = v * 10 + (text[i] - '0');
    if (v > 2147483648ll) return false;  // out of int range (checked again below)
    ++i;
  }
  if (neg) v = -v;
  if (v > 2147483647ll || v < -2147483648ll) return false;
  *out = v;
  *k = i;
  return true;
}

__global__ void k_parse_lines(const char* text, int64_t size, const int64_t* line_begin, int64_t lines, int32_t n,
                              int32_t* pu, int32_t* pv, uint8_t* ok) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= lines) return;
  const int64_t b = line_begin[l];
  const int64_t e = l + 1 < lines ? line_begin[l + 1] : size;  // up to the next line's start
  int64_t k = b, a = 0, c = 0;
  bool good = parse_int(text, e, &k, &a) && parse_int(text, e, &k, &c);
  if (good) {
    a -= 1;
    c -= 1;
    good = a >= 0 && a < n && c >= 0 && c < n && a != c;
  }
  ok[l] = good ? 1 : 0;
  pu[l] = (int32_t)a;
  pv[l] = (int32_t)c;
}

__global__ void k_keep_lines(const int32_t* pu, const int32_t* pv, const uint8_t* ok, const int64_t* pos,
                             int64_t lines, int32_t* u, int32_t* v) {
  const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= lines || !ok[l]) return;
  u[pos[l]] = pu[l];
  v[pos[l]] = pv[l];
}

}  // namespace

// Parses the file into c->bu / c->bv (0-based, valid lines in file order) and
// returns the count.
int64_t parse_batch_file_device(mf_ctx* c, const char* path) {
  cudaStream_t s = c->stream;
  FILE* f = std::fopen(path, "rb");
  if (!f) MF_FAIL(MF_EIO, std::string("could not open ") + path);
  std::fseek(f, 0, SEEK_END);
  const long fsize = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  const int64_t size = fsize > 0 ? (int64_t)fsize : 0;
  std::vector<char> host((size_t)std::max<int64_t>(size, 1));
  const size_t got = size > 0 ? std::fread(host.data(), 1, (size_t)size, f) : 0;
  std::fclose(f);
  if ((int64_t)got != size) MF_FAIL(MF_EIO, std::string("could not read ") + path);
  if (size == 0) return 0;
  DBuf<char> text;
  DBuf<uint8_t> flags;
  DBuf<int64_t> pos, begin;
  text.reserve(size);
  flags.reserve(size);
  pos.reserve(size + 1);
  MF_CUDA(cudaMemcpyAsync(text.p, host.data(), (size_t)size, cudaMemcpyHostToDevice, s));
  MF_K(k_line_starts<<<grid_for(size), kTB, 0, s>>>(text.p, size, flags.p));
  scan_exclusive_u8(flags.p, pos.p, size, c->ws, s);
  int64_t lines = 0;
  MF_CUDA(cudaMemcpyAsync(&lines, pos.p + size, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  begin.reserve(std::max<int64_t>(lines, 1));
  MF_K(k_line_offsets<<<grid_for(size), kTB, 0, s>>>(flags.p, pos.p, size, begin.p));
  DBuf<int32_t> pu, pv;
  pu.reserve(std::max<int64_t>(lines, 1));
  pv.reserve(std::max<int64_t>(lines, 1));
  // flags now holds per-line validity, pos the compaction positions
  MF_K(k_parse_lines<<<grid_for(lines), kTB, 0, s>>>(text.p, size, begin.p, lines, c->n, pu.p, pv.p, flags.p));
  scan_exclusive_u8(flags.p, pos.p, lines, c->ws, s);
  int64_t m = 0;
  MF_CUDA(cudaMemcpyAsync(&m, pos.p + lines, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MF_CUDA(cudaStreamSynchronize(s));
  c->bu.reserve(std::max<int64_t>(m, 1));
  c->bv.reserve(std::max<int64_t>(m, 1));
  c->bins.reserve(std::max<int64_t>(m, 1));
  MF_K(k_keep_lines<<<grid_for(lines), kTB, 0, s>>>(pu.p, pv.p, flags.p, pos.p, lines, c->bu.p, c->bv.p));
  MF_CUDA(cudaGetLastError());
  MF_CUDA(cudaStreamSynchronize(s));
  text.release();
  flags.release();
  pos.release();
  begin.release();
  pu.release();
  pv.release();
  return m;
}

}  // namespace mf
