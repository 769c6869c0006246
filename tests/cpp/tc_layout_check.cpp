// Host check of the tensor-core tile layout (sg-emtf_gb300/csrc/emt_internal.h):
// for island shapes across the supported range, every MMA of the rotation
// reads inside the launch's shared memory, every TMA copy of Q lands inside
// the B region, and the shapes a handle accepts stay within the shared-memory
// limit.  Built and run by tests/test_tc_layout.py.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "emt_internal.h"

int main() {
  const int dims[] = {1, 2, 5, 8, 9, 16, 17, 31, 32, 33, 48, 50, 57, 63, 64, 65, 72, 96, 100, 127, 128};
  const int pops[] = {4, 8, 12, 16, 32, 40, 48, 60, 64, 65, 68, 100, 128};
  long checked = 0, refused = 0, bad = 0;
  for (int bf = 0; bf < 2; ++bf) {
    const bool bf16 = bf != 0;
    // one-island handles, and two-island handles whose widest island sets Np and Kp
    for (int D : dims)
      for (int NP : pops)
        for (int D2 : {0, 1, 64, 128})
          for (int NP2 : {4, 128}) {
            std::vector<std::pair<int, int>> isl{{D, NP}};
            if (D2) isl.push_back({D2, NP2});
            int dmax = 1;
            for (auto& i : isl) dmax = std::max(dmax, i.first);
            const int np = std::max(64, emt::round8(dmax));
            const int kp = bf16 ? emt::round64(dmax) : emt::round32(dmax);
            size_t smem = 0;
            for (auto& i : isl) smem = std::max(smem, emt::tc_layout(i.first, i.second, np, kp, bf16).total);
            if (smem > emt::kSmemLimit) {  // the host refuses such a handle
              ++refused;
              continue;
            }
            for (auto& i : isl) {
              ++checked;
              if (!emt::tc_island_reads_inside(i.first, i.second, np, kp, bf16, smem)) {
                ++bad;
                std::printf("outside: bf16=%d D=%d NP=%d (handle Np=%d Kp=%d smem=%zu)\n", bf ? 1 : 0,
                            i.first, i.second, np, kp, smem);
              }
            }
          }
  }
  // the config-2 islands must be accepted in both forms
  for (int bf = 0; bf < 2; ++bf)
    if (!emt::tc_island_reads_inside(50, 64, 64, bf ? 64 : 64, bf != 0,
                                     emt::tc_layout(50, 64, 64, 64, bf != 0).total)) {
      ++bad;
      std::printf("config-2 island refused (bf16=%d)\n", bf);
    }
  std::printf("checked %ld islands, %ld handles over the shared-memory limit, %ld outside\n", checked,
              refused, bad);
  return bad == 0 ? 0 : 1;
}
