// misfit_main.cpp -- drop-in replacements for the reference's `misfit` and
// `misfit_async` binaries on top of libmisfit_gb.
//
// Same 5 positional arguments (src/misfit/misfit.cu:737-743,
// core/cli_setup.h:28-41), same inputs and outputs:
//   * batch files: every regular file of the folder, ordered by the integer
//     value of its stem, the first <num_batches> parsed (on the device) before
//     any batch runs, each line's insert/delete flag taken against the base
//     graph (src/misfit/misfit.cu:802-828);
//   * final MIS written 1-based to datasets/Final_MISs/<stem>_flash_final_mis.txt
//     under the current directory (src/misfit/misfit.cu:892-907);
//   * end-of-run compaction over the input .egr unless
//     MISFIT_SKIP_COMPACTION=1 (src/misfit/misfit.cu:909-926);
//   * the stdout lines harnesses parse ("Processing batch i/N | Edges: X",
//     "Total Batch Time:", "Batch i/N | edges=X | time=Y ms",
//     "Total processing time:", "Final MIS cardinality:").
// Errors print one line to stderr and return 1 (the reference exits 1 too).
// Built twice: misfit (sync) and misfit_async (-DMISFIT_ASYNC=1, printing the
// pipelined engine's per-batch line, core/reporting.h:29-36).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "misfit_gb.h"

namespace {

int fail(const char* what, int status) {
  std::cerr << "ERROR: " << what << ": " << mf_status_string(status) << " - " << mf_last_error() << std::endl;
  return 1;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Batch {
  std::vector<int32_t> u, v;
  std::vector<uint8_t> ins;
};

}  // namespace

int main(int argc, char** argv) {
#ifdef MISFIT_ASYNC
  const bool async_engine = true;
#else
  const bool async_engine = false;
#endif
  if (argc < 6) {
    std::cerr << "Usage: " << argv[0] << " <graph.egr> <initial_mis.txt> <batch_folder> <num_batches> <gpu_device_id>"
              << std::endl;
    return 1;
  }
  const std::string graph_path = argv[1];
  int num_batches = 0, gpu = 0;
  try {
    num_batches = std::stoi(argv[4]);
    gpu = std::stoi(argv[5]);
  } catch (...) {
    std::cerr << "ERROR: <num_batches> and <gpu_device_id> must be integers" << std::endl;
    return 1;
  }
  std::cout << "=========================================START=====================================================" << std::endl;
  std::cout << (async_engine ? "======================================= MISFIT_Async (PIPELINED, GB300) ========================================="
                             : "======================================= MISFIT (SYNC, GB300) =========================================")
            << std::endl;
  if (graph_path.size() < 4 || graph_path.substr(graph_path.size() - 4) != ".egr")
    std::cerr << "[Warning] " << graph_path << " does not end in .egr" << std::endl;

  const double setup0 = now_ms();
  mf_ctx* ctx = nullptr;
  int st = mf_open_egr(graph_path.c_str(), gpu, &ctx);
  if (st != MF_OK) return fail("opening the graph", st);
  int32_t n = 0;
  mf_num_nodes(ctx, &n);
  int64_t max_csr = 0;
  mf_get_max_csr(ctx, &max_csr);
  std::cout << "MAX_CSR_ELEMENTS set to: " << max_csr << std::endl;

  std::vector<uint8_t> mis((size_t)n, 0);
  int64_t initial_card = 0;
  st = mf_read_mis_file(argv[2], n, mis.data(), &initial_card);
  if (st != MF_OK) return fail("reading the initial MIS", st);
  st = mf_set_mis(ctx, mis.data(), n);
  if (st != MF_OK) return fail("uploading the initial MIS", st);
  std::cout << "Initial MIS cardinality: " << initial_card << std::endl;

  // every batch is parsed and flagged against the base graph before any runs
  char* names = nullptr;
  int64_t nfiles = 0;
  st = mf_list_batch_files(argv[3], &names, &nfiles);
  if (st != MF_OK) return fail("listing the batch folder", st);
  std::vector<std::string> files;
  {
    std::istringstream is(names);
    std::string line;
    while (std::getline(is, line))
      if (!line.empty()) files.push_back(line);
  }
  mf_free(names);
  std::vector<Batch> batches;
  for (const auto& f : files) {
    if ((int)batches.size() >= num_batches) break;
    const std::string path = (std::filesystem::path(argv[3]) / f).string();
    // parsed and flagged on the device, against the base graph (no batch has run yet)
    int32_t *u = nullptr, *v = nullptr;
    uint8_t* ins = nullptr;
    int64_t m = 0;
    st = mf_parse_batch_file(ctx, path.c_str(), &u, &v, &ins, &m);
    if (st != MF_OK) return fail("reading a batch file", st);
    Batch b;
    b.u.assign(u, u + m);
    b.v.assign(v, v + m);
    b.ins.assign(ins, ins + m);
    mf_free(u);
    mf_free(v);
    mf_free(ins);
    batches.push_back(std::move(b));
  }
  const int nb = (int)batches.size();
  const double setup_ms = now_ms() - setup0;

  double time_cum = 0.0;
  int64_t total_updates = 0;
  if (!async_engine) {
    for (int i = 0; i < nb; ++i) {
      const Batch& b = batches[(size_t)i];
      const int64_t m = (int64_t)b.u.size();
      std::cout << "\n" << std::string(60, '=') << std::endl;
      std::cout << "Processing batch " << (i + 1) << "/" << nb << " | Edges: " << m << std::endl;
      const double t0 = now_ms();
      st = mf_apply_batch(ctx, b.u.data(), b.v.data(), b.ins.data(), m);
      if (st != MF_OK) return fail("processing a batch", st);
      const double dt = now_ms() - t0;
      time_cum += dt;
      total_updates += m;
      mf_batch_stats bs{};
      mf_last_batch_stats(ctx, &bs);
      std::cout << std::fixed << std::setprecision(3);
      std::cout << "=== BATCH TIMING BREAKDOWN ===" << std::endl;
      std::cout << "Total Batch Time: " << dt << " ms\n" << std::endl;
      std::cout << "  Device time:             " << bs.device_ms << " ms (GPU)" << std::endl;
      std::cout << "  Sub-batches:             " << bs.sub_batches << std::endl;
      std::cout << "  Cluster count:           " << bs.clusters << std::endl;
    }
  } else {
    // The pipelined loop of misfit_async (src/misfit_async/misfit_async.cu:826-876):
    // batch i+1 is launched before batch i is collected; a batch's time runs
    // from its launch to its collection, and the total is the loop's wall time.
    std::vector<double> launched((size_t)nb, 0.0);
    const double wall0 = now_ms();
    auto launch = [&](int i) {
      const Batch& b = batches[(size_t)i];
      launched[(size_t)i] = now_ms();
      return mf_apply_batch_async(ctx, b.u.data(), b.v.data(), b.ins.data(), (int64_t)b.u.size());
    };
    if (nb > 0 && (st = launch(0)) != MF_OK) return fail("launching a batch", st);
    for (int i = 0; i < nb; ++i) {
      const int64_t m = (int64_t)batches[(size_t)i].u.size();
      std::cout << "\n" << std::string(60, '=') << std::endl;
      std::cout << "Processing batch " << (i + 1) << "/" << nb << " | Edges: " << m << std::endl;
      if (i + 1 < nb && (st = launch(i + 1)) != MF_OK) return fail("launching a batch", st);
      mf_batch_stats bs{};
      st = mf_collect(ctx, &bs);
      if (st != MF_OK) return fail("processing a batch", st);
      const double dt = now_ms() - launched[(size_t)i];
      total_updates += m;
      std::cout << std::fixed << std::setprecision(3);
      std::cout << "Batch " << (i + 1) << "/" << nb << " | edges=" << m << " | time=" << dt << "ms"
                << " | clusters=" << bs.clusters << std::endl;
      std::cout << "Total Batch Time: " << dt << " ms\n" << std::endl;
      std::cout << "  Device time:             " << bs.device_ms << " ms (GPU)" << std::endl;
      std::cout << "  Sub-batches:             " << bs.sub_batches << std::endl;
    }
    time_cum = now_ms() - wall0;
  }

  st = mf_get_mis(ctx, mis.data(), n);
  if (st != MF_OK) return fail("reading the final MIS", st);
  int64_t updated_card = 0;
  for (uint8_t x : mis) updated_card += x != 0;
  {
    const std::string out_dir = "datasets/Final_MISs";
    std::error_code ec;
    std::filesystem::create_directories(out_dir, ec);
    const std::string stem = std::filesystem::path(graph_path).stem().string();
    const std::string out = out_dir + "/" + stem + "_flash_final_mis.txt";
    if (mf_write_mis_file(out.c_str(), mis.data(), n) == MF_OK)
      std::cout << "Saved final MIS to " << out << std::endl;
    else
      std::cerr << "Warning: Could not open file to save final MIS: " << out << std::endl;
  }

  const char* skip_env = std::getenv("MISFIT_SKIP_COMPACTION");
  const bool skip = skip_env != nullptr && std::string(skip_env) == "1";
  double compact_ms = 0.0;
  if (!skip) {
    const double c0 = now_ms();
    st = mf_compact(ctx, graph_path.c_str(), 1);
    if (st != MF_OK) return fail("compacting the graph", st);
    compact_ms = now_ms() - c0;
  } else {
    std::cout << "\n[MISFIT_SKIP_COMPACTION=1] Skipping end-of-cycle compaction - on-disk .egr left untouched." << std::endl;
  }
  const int processed = nb == 0 ? 1 : nb;
  std::cout << "\n" << std::string(80, '=') << std::endl;
  std::cout << "=== FINAL RESULTS ===" << std::endl;
  std::cout << std::string(80, '=') << "\n" << std::endl;
  std::cout << "Graph Statistics:" << std::endl;
  std::cout << "  Initial MIS cardinality: " << initial_card << std::endl;
  std::cout << "  Final MIS cardinality:   " << updated_card << std::endl;
  std::cout << "  Cardinality change:      " << std::llabs(initial_card - updated_card) << std::endl;
  std::cout << "  Number of batches:       " << processed << "\n" << std::endl;
  std::cout << "Overall Timing Results:" << std::endl;
  std::cout << std::fixed << std::setprecision(3);
  std::cout << "  Total processing time:   " << time_cum << " milliseconds" << std::endl;
  std::cout << "  Average time per batch:  " << time_cum / processed << " milliseconds" << std::endl;
  std::cout << std::setprecision(1);
  std::cout << "  Processing rate:         " << (time_cum > 0 ? processed / (time_cum / 1000.0) : 0.0)
            << " batches/second" << std::endl;
  std::cout << "  Edge updates/second:     " << (time_cum > 0 ? total_updates / (time_cum / 1000.0) : 0.0) << std::endl;
  std::cout << std::setprecision(3);
  std::cout << "\nEnd-of-cycle compaction time (NOT counted in per-batch numbers above): " << compact_ms << " ms"
            << std::endl;
  if (async_engine) {
    std::cout << "\n=== FINAL SUMMARY ===" << std::endl;
    std::cout << "Setup time:      " << setup_ms << " ms" << std::endl;
    std::cout << "Processing time: " << time_cum << " ms" << std::endl;
    std::cout << "End-to-end time: " << setup_ms + time_cum + compact_ms << " ms" << std::endl;
    std::cout << "Initial MIS size: " << initial_card << std::endl;
    std::cout << "Final MIS size:   " << updated_card << std::endl;
  }
  std::cout << std::string(80, '=') << std::endl;
  mf_close(ctx);
  return 0;
}
