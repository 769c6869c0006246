// emt_records.cpp -- run records, the average normalised objective and the
// reference's output files, on the host over the library's public ABI.
//
// The reference records each task's best fitness at every transfer
// interval plus one "near-worst" value of the initial population
// (proposed model/SG-EMTF_DE.cu:1575,1594-1595,1632, written at :1791-1809;
// the GA file's writer is commented out at SG-EMTF.cu:2015-2026), and its
// analysis tool turns runs of such rows into the average normalised
// objective (data process/源.cpp:122-209).  para.txt (SG-EMTF.cu:244-264) and
// output_0.txt (:1971-1983) hold the instances and the final populations'
// sorted fitness.  The number format is the C++ stream default the reference
// writes with: 6 significant digits, "%g".
#include <algorithm>
#include <climits>
#include <cstdio>
#include <vector>

#include "../../include/sgemtf.h"

namespace {

int task_count(emt_handle_t* h, int32_t* n) {
  emt_stats st;
  const int rc = emt_get_stats(h, &st);
  if (rc) return rc;
  *n = st.n_tasks;
  return EMT_OK;
}

// The reference's type number of a function id (inverse of
// emt_function_from_reference).
int reference_type(int fid) {
  for (int r = 0; r < EMT_NUM_FUNCTIONS; ++r)
    if (emt_function_from_reference(r) == fid) return r;
  return -1;
}

}  // namespace

extern "C" {

EMT_API int emt_record_run(emt_handle_t* h, int32_t generations, int32_t interval, void* stream,
                           float* record) {
  if (!h || !record || generations < 0 || interval < 1 || generations % interval != 0)
    return EMT_ERR_INVALID_ARG;
  int32_t n = 0;
  int rc = task_count(h, &n);
  if (rc) return rc;
  const int P = generations / interval, cols = P + 2;
  std::vector<float> best((size_t)std::max(n, 1));
  if ((rc = emt_get_best_all(h, best.data()))) return rc;
  for (int t = 0; t < n; ++t) record[(size_t)t * cols] = best[t];
  // the near-worst of the population on entry: the first member of the last
  // 32-member bank of the ascending order
  std::vector<float> fit;
  for (int t = 0; t < n; ++t) {
    int32_t pop = 0;
    if ((rc = emt_get_task_info(h, t, nullptr, nullptr, &pop))) return rc;
    fit.resize((size_t)pop);
    if ((rc = emt_get_population(h, t, nullptr, fit.data()))) return rc;
    std::sort(fit.begin(), fit.end());
    record[(size_t)t * cols + P + 1] = fit[(size_t)(32 * ((pop - 1) / 32))];
  }
  for (int c = 1; c <= P; ++c) {
    if ((rc = emt_run(h, interval, stream))) return rc;
    if ((rc = emt_get_best_all(h, best.data()))) return rc;
    for (int t = 0; t < n; ++t) record[(size_t)t * cols + c] = best[t];
  }
  return EMT_OK;
}

EMT_API int emt_write_record(const char* path, int32_t tasks, int32_t cols, const float* record) {
  if (!path || tasks < 0 || cols < 1 || (tasks > 0 && !record)) return EMT_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "a");
  if (!f) return EMT_ERR_INVALID_ARG;
  for (int t = 0; t < tasks; ++t) {
    for (int c = 0; c < cols; ++c) std::fprintf(f, "%g ", (double)record[(size_t)t * cols + c]);
    std::fputc('\n', f);
  }
  std::fputc('\n', f);
  return std::fclose(f) == 0 ? EMT_OK : EMT_ERR_INVALID_ARG;
}

EMT_API int emt_ano(int32_t runs, int32_t tasks, int32_t cols, const float* records, float* ano) {
  if (runs < 1 || tasks < 1 || cols < 2 || !records || !ano) return EMT_ERR_INVALID_ARG;
  const int P = cols - 1;  // recording points; column P is the near-worst
  auto at = [&](int k, int i, int j) { return records[((size_t)k * tasks + i) * cols + j]; };
  std::vector<float> result((size_t)P, 0.f);
  for (int i = 0; i < tasks; ++i) {
    // the tool's sentinels: INT_MAX as a float and -1
    float mn = (float)INT_MAX, mx = -1.f;
    for (int k = 0; k < runs; ++k) {
      if (at(k, i, P - 1) < mn) mn = at(k, i, P - 1);
      if (at(k, i, P) > mx) mx = at(k, i, P);
    }
    for (int j = 0; j < P; ++j)
      for (int k = 0; k < runs; ++k) {
        float v = 0.f;
        if (mx - mn != 0.f) v = (at(k, i, j) - mn) / (mx - mn);
        result[j] += v;
      }
  }
  for (int j = 0; j < P; ++j) ano[j] = result[j] / (float)(tasks * runs);
  return EMT_OK;
}

EMT_API int emt_write_fitness(emt_handle_t* h, const char* path) {
  if (!h || !path) return EMT_ERR_INVALID_ARG;
  int32_t n = 0;
  int rc = task_count(h, &n);
  if (rc) return rc;
  std::vector<std::vector<float>> fit((size_t)n);
  for (int t = 0; t < n; ++t) {
    int32_t pop = 0;
    if ((rc = emt_get_task_info(h, t, nullptr, nullptr, &pop))) return rc;
    fit[t].resize((size_t)pop);
    if ((rc = emt_get_population(h, t, nullptr, fit[t].data()))) return rc;
    std::sort(fit[t].begin(), fit[t].end());
  }
  FILE* f = std::fopen(path, "a");
  if (!f) return EMT_ERR_INVALID_ARG;
  for (const auto& v : fit) {
    for (float x : v) std::fprintf(f, "%g ", (double)x);
    std::fputc('\n', f);
  }
  std::fputc('\n', f);
  return std::fclose(f) == 0 ? EMT_OK : EMT_ERR_INVALID_ARG;
}

EMT_API int emt_write_para(emt_handle_t* h, const char* path) {
  if (!h || !path) return EMT_ERR_INVALID_ARG;
  int32_t n = 0;
  int rc = task_count(h, &n);
  if (rc) return rc;
  std::vector<std::vector<float>> M((size_t)n), b((size_t)n);
  std::vector<int> types((size_t)n);
  std::vector<float> Q, o;
  for (int t = 0; t < n; ++t) {
    int32_t fid = 0, D = 0;
    if ((rc = emt_get_task_info(h, t, &fid, &D, nullptr))) return rc;
    Q.resize((size_t)D * D);
    o.resize((size_t)D);
    if ((rc = emt_get_task_params(h, t, Q.data(), o.data()))) return rc;
    for (int r = 0; r < D; ++r)
      for (int c = 0; c < D; ++c)
        if (r != c && Q[(size_t)r * D + c] != 0.f) return EMT_ERR_UNSUPPORTED;
    for (int d = 0; d < D; ++d) {
      M[t].push_back(Q[(size_t)d * D + d]);
      b[t].push_back(0.f - o[d]);  // b = -o, without a signed zero
    }
    types[t] = reference_type(fid);
  }
  FILE* f = std::fopen(path, "w");
  if (!f) return EMT_ERR_INVALID_ARG;
  for (int t = 0; t < n; ++t) {
    for (size_t d = 0; d < M[t].size(); ++d)
      std::fprintf(f, "%g %g ", (double)M[t][d], (double)b[t][d]);
    std::fputc('\n', f);
  }
  std::fputc('\n', f);
  for (int t = 0; t < n; ++t) std::fprintf(f, "%d ", types[t]);
  std::fputc('\n', f);
  return std::fclose(f) == 0 ? EMT_OK : EMT_ERR_INVALID_ARG;
}

}  // extern "C"
