// host_example.cpp -- a C++ host program driving the engine through the C ABI
// only (include/sgemtf.h), the way a maintainer replaces the reference's
// iter() threads (proposed model/SG-EMTF.cu:1646-1723, 1839-1915) and its
// initialization() globals (:293-380).  Built with g++ by
// tests/test_gpu_cpp_host.py, which feeds it a task file and compares its
// output with the same run through the Python binding.
//
// usage: host_example <tasks.bin> <out.bin>
//   tasks.bin: int32 T, D, NP, generations, epoch; T int32 reference type
//              ids (SG-EMTF.cu:917-1101 numbering); T*D float M; T*D float b
//   out.bin:   T float best FP32 fitness, then task 0's population (NP*D)
#include <cstdint>
#include <cstdio>
#include <vector>

#include "sgemtf.h"

static bool read_all(FILE* f, void* p, size_t bytes) { return fread(p, 1, bytes, f) == bytes; }

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s tasks.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE* in = fopen(argv[1], "rb");
  if (!in) return 2;
  int32_t hdr[5];
  if (!read_all(in, hdr, sizeof(hdr))) return 2;
  const int T = hdr[0], D = hdr[1], NP = hdr[2], gens = hdr[3], epoch = hdr[4];
  std::vector<int32_t> ref_type(T);
  std::vector<float> M((size_t)T * D), b((size_t)T * D);
  if (!read_all(in, ref_type.data(), sizeof(int32_t) * T) ||
      !read_all(in, M.data(), sizeof(float) * M.size()) ||
      !read_all(in, b.data(), sizeof(float) * b.size()))
    return 2;
  fclose(in);

  emt_config cfg;
  emt_config_default(&cfg);
  // the reference GA (SG-EMTF.cu:44-49): SBX eta 2, PM eta 5 on every gene
  cfg.algorithm = EMT_GA_SBX_PM;
  cfg.eta_c = 2.f;
  cfg.p_c = 1.f;
  cfg.eta_m = 5.f;
  cfg.p_m = 1.f;
  cfg.transfer_interval = epoch;       // INTERVAL_TRANSFER (:36)
  cfg.transfer_rate = 50.f / 512.f;    // TRANSFER_NUM / INDIVNUM (:29,38)
  cfg.transfer_mix = 0.4f;             // 1 - CROSSOVER_RATE (:45, used at :1551)
  cfg.flags = EMT_FLAG_REF_BOXES | EMT_FLAG_REF_GRIEWANK_NO_PRODUCT |
              EMT_FLAG_REF_WEIERSTRASS_CONST | EMT_FLAG_REF_ACKLEY_E;
  cfg.seed = 12345;

  emt_handle_t* h = nullptr;
  int rc = emt_create(&cfg, &h);
  if (rc != EMT_OK) {
    fprintf(stderr, "emt_create: %s\n", emt_status_string(rc));
    return 1;
  }
  // the reference's z = M[d] * (x + b[d]) is EMT_ROTATION_DIAG with o = -b
  std::vector<float> negb(b.size());
  for (size_t i = 0; i < b.size(); ++i) negb[i] = -b[i];
  std::vector<emt_task_desc> tasks(T);
  for (int t = 0; t < T; ++t)
    tasks[t] = emt_task_desc{emt_function_from_reference(ref_type[t]), D, NP, 0.f, 0.f,
                             EMT_ROTATION_DIAG, nullptr, M.data() + (size_t)t * D,
                             negb.data() + (size_t)t * D};
  if (emt_add_tasks(h, T, tasks.data()) != EMT_OK) {
    fprintf(stderr, "emt_add_tasks: %s\n", emt_last_error(h));
    return 1;
  }
  void* stream = nullptr;  // the legacy default stream; any cudaStream_t works
  for (int g = 0; g < gens; g += epoch)
    if (emt_run(h, epoch, stream) != EMT_OK) {
      fprintf(stderr, "emt_run: %s\n", emt_last_error(h));
      return 1;
    }
  if (emt_sync(h) != EMT_OK) {
    fprintf(stderr, "emt_sync: %s\n", emt_last_error(h));
    return 1;
  }
  std::vector<float> best(T), pop((size_t)NP * D), fit(NP);
  if (emt_get_best_all(h, best.data()) != EMT_OK ||
      emt_get_population(h, 0, pop.data(), fit.data()) != EMT_OK) {
    fprintf(stderr, "read-back: %s\n", emt_last_error(h));
    return 1;
  }
  emt_destroy(h);
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 2;
  fwrite(best.data(), sizeof(float), best.size(), out);
  fwrite(pop.data(), sizeof(float), pop.size(), out);
  fclose(out);
  printf("ok %d tasks, %d generations\n", T, gens);
  return 0;
}
