// emt_cvrp.cu -- CVRP multitask engine: one island of permutations per
// instance, decoded by Prins' split, exact int32 costs.
//
// The reference's CVRP variant (proposed model/SG-EMTF_cvrp.cu, per-task
// host function iter() at :1487-1607, params {dimension, cars, customers} at
// :1496-1500) encodes a giant tour with zero separators and is unfinished
// (its crossover overwrites every gene with 1, :731-736).  This engine keeps
// its interface shape (one island per instance, periodic knowledge transfer)
// and implements the published methods:
//   - giant tour of customers 1..n, split into capacity-feasible routes by
//     the shortest-path procedure of Prins (Comput. Oper. Res. 31, 2004);
//   - binary tournaments, order crossover (Davis 1985), swap and 2-opt
//     (segment reversal) mutation; child i replaces member i when its cost is
//     not worse (the reference's selection rule, SG-EMTF.cu:752-769);
//   - elite transfer of whole permutations between instances with the same
//     customer count (knowledgeTransfer, SG-EMTF.cu:1514-1591).
// All arithmetic is integer, so every cost and every population matches the
// host replay bit for bit.
//
// Kernel layout: one CTA per instance, one thread per member; shared memory
// holds the node table {x, y, distance to depot, demand}, the island and its
// children, and each thread's split deque.  Distances between customers are
// recomputed exactly from the integer coordinates where the split needs them
// (no (n+1)^2 matrix on the device), which keeps three CTAs per SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <type_traits>
#include <string>
#include <vector>

#include "../../include/sgemtf.h"
#include "emt_common.cuh"

namespace emt {
namespace cvrp {

enum : uint32_t {
  P_NODE = 16, P_POP_INIT = 17, P_SELECT = 18, P_OX = 19, P_MUTATE = 20, P_PARTNER = 21
};

struct InstDev {
  int32_t n, capacity;
  int64_t node_off;  // int4 {x, y, d0, demand}, n+1 entries
  int64_t pop_off;   // uint8, NP*n
  int32_t cost_off;  // int32, NP
  int32_t pad;
  int64_t elite_off; // uint8, NP*n per buffer
};

struct Args {
  const InstDev* inst;
  int32_t n_inst, NP, gens, mode;  // mode: 0 epoch, 1 init
  int32_t ring;                    // deque slots per thread (a multiple of 4)
  int32_t used_words;              // words of the per-thread crossover bitmap
  const int4* node;
  uint8_t* pop;
  int32_t* cost;
  uint32_t* gen;
  uint64_t seed;
  float p_cross, p_swap, p_2opt, transfer_rate;
  int32_t transfer_import, transfer_export;
  const uint8_t* elites_in;
  uint8_t* elites_out;
  unsigned long long* stats;  // [0] evaluations [1] transfers accepted [2] migrants accepted
  int32_t* err;
  size_t smem_bytes;
  // sub-islands: groups per island (1 = none), migration interval and count
  int32_t subislands, mig_interval, mig_count;
};

__host__ __device__ inline size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// Shared memory of one instance's CTA (P = threads of the block, R = deque
// slots per thread, QB = bytes of a stored demand prefix, UW = bitmap words).
// Per-thread arrays are interleaved [slot][thread] so that a warp's accesses
// fall in 32 distinct banks whatever slot each lane is at (sub-word demand
// prefixes: each lane owns one word per 4 / QB slots).  Member i's tour lives
// in pool row (cur[i] * P + i); its child is built in the other row and
// accepted by flipping cur[i].  The rank list shares the child-cost array:
// ranks are only needed outside the generation loop.
struct Layout {
  size_t node, pool, cost, kcost, cur, used, ringA, ringQ, total;
};

__host__ __device__ inline Layout layout(int n, int P, int R, int QB, int UW) {
  Layout L;
  size_t off = 0;
  L.node = off;  off = align16(off + sizeof(int4) * (n + 1));
  L.pool = off;  off = align16(off + (size_t)2 * P * n);
  L.cost = off;  off = align16(off + sizeof(int32_t) * P);
  L.kcost = off; off = align16(off + sizeof(int32_t) * P);
  L.cur = off;   off = align16(off + (size_t)P);
  L.used = off;  off = align16(off + sizeof(uint32_t) * (size_t)UW * P);
  L.ringA = off; off = align16(off + sizeof(int32_t) * (size_t)R * P);
  L.ringQ = off; off = align16(off + (size_t)QB * R * P);
  L.total = off;
  return L;
}

// The evaluation kernel's shared memory: the instance and the deque rings only.
__host__ __device__ inline Layout eval_layout(int n, int P, int R, int QB) {
  Layout L{};
  size_t off = 0;
  L.node = off;  off = align16(off + sizeof(int4) * (n + 1));
  L.ringA = off; off = align16(off + sizeof(int32_t) * (size_t)R * P);
  L.ringQ = off; off = align16(off + (size_t)QB * R * P);
  L.total = off;
  return L;
}

// Demand prefixes Q_i in the deque, stored in QB bytes.  Every difference
// the split tests, Q_j - Q_i for i in the deque, lies in [0, 2 * capacity]
// (the entry was inside the previous window, plus one demand), so storing Q_i
// modulo 2^(8 QB) and masking the difference is exact when 2 * capacity <
// 2^(8 QB).  The host picks QB from the largest capacity.
template <int QB>
struct QRing {
  using T = typename std::conditional<QB == 1, uint8_t,
            typename std::conditional<QB == 2, uint16_t, int32_t>::type>::type;
  T* base;  // this lane's first element
  int P;
  __device__ __forceinline__ QRing(unsigned char* region, int lane, int P_) : P(P_) {
    base = (T*)region + lane * (4 / QB);
  }
  __device__ __forceinline__ int idx(int slot) const {
    return QB == 4 ? slot * P : (slot / (4 / QB)) * (4 / QB) * P + (slot % (4 / QB));
  }
  __device__ __forceinline__ void put(int slot, int32_t q) { base[idx(slot)] = (T)q; }
  __device__ __forceinline__ int32_t get(int slot) const { return (int32_t)base[idx(slot)]; }
  // Q - stored, exact under the capacity bound above
  static __device__ __forceinline__ int32_t gap(int32_t Q, int32_t stored) {
    return QB == 4 ? Q - stored : (int32_t)((uint32_t)(Q - stored) & ((1u << (8 * QB)) - 1u));
  }
};

constexpr int kMaxN = 255;

// Rounded Euclidean distance round(sqrt(dx^2 + dy^2)) of integer points
// with coordinates in [0, 40000], exact: r0 = trunc(sqrt(v)) from a floating
// square root (within 1 of floor(sqrt(v)) for v < 2^32: relative error below
// 2^-21 on values below 2^16), one integer correction each way, then
// sqrt(v) < r + 1/2 <=> v <= r^2 + r.  Host and device give the same bits.
EMT_HD uint32_t round_dist(int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
  const int32_t dx = x0 - x1, dy = y0 - y1;
  const uint32_t v = (uint32_t)(dx * dx) + (uint32_t)(dy * dy);  // <= 3.2e9
#if defined(__CUDA_ARCH__)
  const float f = (float)v;
  uint32_t r = v ? (uint32_t)(f * rsqrtf(f)) : 0u;
#else
  uint32_t r = (uint32_t)std::sqrt((double)v);
#endif
  if (r * r > v)
    --r;
  else if ((r + 1u) * (r + 1u) <= v)
    ++r;
  return v <= r * r + r ? r : r + 1u;
}

// Split of one giant tour p_0..p_{n-1} into capacity-feasible routes, the
// shortest-path procedure of Prins (Comput. Oper. Res. 31, 2004) evaluated in
// O(n) with the monotone-deque form of Vidal (Comput. Oper. Res. 69, 2016).
// With S_k = sum_{m<k} d(p_m, p_{m+1}) and Q_k = sum_{m<k} q(p_m), the route
// serving p_i..p_{j-1} costs d0(p_i) - S_i + S_{j-1} + d0(p_{j-1}), so
//   V_j = S_{j-1} + d0(p_{j-1}) + min { A_i : i < j, Q_j - Q_i <= capacity },
//   A_i = V_i + d0(p_i) - S_i.
// The deque holds candidate i in increasing i and increasing A_i; its front
// is the minimum, kept in registers.  All integer, so V_n equals the
// label-correcting form exactly.  A window holds at most Lmax + 1 entries
// (Lmax = most customers one route can serve), which the R-slot ring covers;
// rA points at this thread's slot 0, slots P apart.
template <int QB>
__device__ __forceinline__ int32_t split_linear(int n, const int4* __restrict__ node,
                                                int32_t capacity, const uint8_t* __restrict__ perm,
                                                int32_t* __restrict__ rA, QRing<QB> rQ, int P,
                                                int R) {
  int head = 0, tail = 0, cnt = 0;  // ring positions in [0, R), entries head .. tail - 1
  int32_t V = 0, S = 0, Q = 0, fA = 0, fQ = 0;
  int32_t px = 0, py = 0;
  for (int j = 1; j <= n; ++j) {
    const int4 nd = node[perm[j - 1]];  // x, y, d0, demand
    if (j > 1) S += (int32_t)round_dist(px, py, nd.x, nd.y);
    px = nd.x;
    py = nd.y;
    const int32_t A = V + nd.z - S;
    while (cnt > 0) {
      const int b = tail == 0 ? R - 1 : tail - 1;
      if (rA[b * P] < A) break;
      tail = b;
      --cnt;
    }
    if (cnt == 0) {
      fA = A;
      fQ = Q;
    }
    rA[tail * P] = A;
    rQ.put(tail, Q);
    tail = tail + 1 == R ? 0 : tail + 1;
    ++cnt;
    Q += nd.w;
    // the newest candidate (i = j - 1) always fits: q(p_{j-1}) <= capacity
    while (QRing<QB>::gap(Q, fQ) > capacity && cnt > 1) {
      head = head + 1 == R ? 0 : head + 1;
      --cnt;
      fA = rA[head * P];
      fQ = rQ.get(head);
    }
    V = S + nd.z + fA;
  }
  return V;
}

__device__ __forceinline__ int better(const int32_t* cost, int a, int b) {
  return (cost[a] < cost[b] || (cost[a] == cost[b] && a <= b)) ? a : b;
}

__device__ __forceinline__ void report(int32_t* err, int32_t code) {
  if (err) atomicCAS(err, 0, code);
}

// byrank[r] = member of rank r by (cost, index).
__device__ void rank_members(const int32_t* cost, int NP, int32_t* byrank) {
  for (int i = threadIdx.x; i < NP; i += blockDim.x) {
    const int32_t ci = cost[i];
    int r = 0;
    for (int j = 0; j < NP; ++j) r += (cost[j] < ci || (cost[j] == ci && j < i)) ? 1 : 0;
    byrank[r] = i;
  }
  __syncthreads();
}

// The instance's node table into shared memory.
__device__ void load_instance(const Args& a, const InstDev& d, int4* node) {
  for (int it = threadIdx.x; it <= d.n; it += blockDim.x) node[it] = a.node[d.node_off + it];
}

template <int QB>
__global__ void __launch_bounds__(256) cvrp_epoch_kernel(const Args a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int t = blockIdx.x;
  if (t >= a.n_inst) return;
  const InstDev d = a.inst[t];
  const int n = d.n, NP = a.NP, P = blockDim.x;
  if (n < 1 || n > kMaxN || NP < 2 || NP > P) {
    if (threadIdx.x == 0) report(a.err, 1);
    return;
  }
  const Layout L = layout(n, P, a.ring, QB, a.used_words);
  if (L.total > a.smem_bytes || n >= 32 * a.used_words) {
    if (threadIdx.x == 0) report(a.err, 2);
    return;
  }
  int4* node = (int4*)(smem + L.node);
  uint8_t* pool = smem + L.pool;
  int32_t* cost = (int32_t*)(smem + L.cost);
  int32_t* kcost = (int32_t*)(smem + L.kcost);
  uint8_t* cur = smem + L.cur;
  uint32_t* used = (uint32_t*)(smem + L.used) + threadIdx.x;
  int32_t* byrank = kcost;
  int32_t* rA = (int32_t*)(smem + L.ringA) + threadIdx.x;
  const QRing<QB> rQ(smem + L.ringQ, threadIdx.x, P);
  const int R = a.ring, UW = a.used_words;
  auto row = [&](int m, int s) { return pool + (size_t)(s * P + m) * n; };

  load_instance(a, d, node);
  const int i = threadIdx.x;
  uint8_t* gpop = a.pop + d.pop_off;
  if (a.mode == 1) {
    if (i < NP) {
      cur[i] = 0;
      uint8_t* q = row(i, 0);
      for (int k = 0; k < n; ++k) q[k] = (uint8_t)(k + 1);
      U4 w{0, 0, 0, 0};
      for (int k = n - 1, s = 0; k > 0; --k, ++s) {
        if ((s & 3) == 0) w = draw(a.seed, (uint32_t)t, 0u, (uint32_t)i, P_POP_INIT, (uint32_t)(s >> 2));
        const int j = (int)(word(w, s & 3) % (uint32_t)(k + 1));
        const uint8_t tmp = q[k];
        q[k] = q[j];
        q[j] = tmp;
      }
    }
    __syncthreads();
    if (i < NP) cost[i] = split_linear(n, node, d.capacity, row(i, 0), rA, rQ, P, R);
    if (threadIdx.x == 0) {
      a.gen[t] = 0;
      if (a.stats) atomicAdd(a.stats + 0, (unsigned long long)NP);
    }
  } else {
    for (int it = threadIdx.x; it < NP * n; it += blockDim.x) pool[it] = gpop[it];  // rows (0, m)
    for (int it = threadIdx.x; it < NP; it += blockDim.x) {
      cost[it] = a.cost[d.cost_off + it];
      cur[it] = 0;
    }
    __syncthreads();
    const uint32_t gen0 = a.gen[t];
    // ---- elite transfer in ----
    if (a.transfer_import && a.elites_in && a.n_inst > 1) {
      const U4 w = draw(a.seed, (uint32_t)t, gen0, 0u, P_PARTNER, 0);
      uint32_t p = w.x % (uint32_t)(a.n_inst - 1);
      if (p >= (uint32_t)t) ++p;
      const InstDev pd = a.inst[p];
      if (pd.n == n) {  // permutations transfer between equal customer counts
        rank_members(cost, NP, byrank);
        int k = (int)(a.transfer_rate * (float)NP + 0.5f);
        k = k < 1 ? 1 : (k > NP ? NP : k);
        const uint8_t* el = a.elites_in + pd.elite_off;
        // candidate c goes to the spare row of the member of rank NP - k + c
        for (int it = threadIdx.x; it < k * n; it += blockDim.x) {
          const int c = it / n, q = it - c * n;
          row(byrank[NP - k + c], 1)[q] = el[it];
        }
        __syncthreads();
        int acc = 0;
        if (i < k) {
          const int m = byrank[NP - k + i];
          const int32_t cc = split_linear(n, node, d.capacity, row(m, 1), rA, rQ, P, R);
          if (cc < cost[m]) {
            cur[m] = 1;
            cost[m] = cc;
            acc = 1;
          }
        }
        if (acc && a.stats) atomicAdd(a.stats + 1, 1ull);
        if (threadIdx.x == 0 && a.stats) atomicAdd(a.stats + 0, (unsigned long long)k);
        __syncthreads();
      }
    }
    // ---- generations ----
    const int S = a.subislands > 1 ? a.subislands : 1, NPs = NP / S;
    for (int g = 0; g < a.gens; ++g) {
      const uint32_t G = gen0 + (uint32_t)g + 1u;
      // ring migration between the sub-islands (IslandMigration,
      // SG-EMTF_cvrp.cu:965-1020): before generation G when due, the r-th
      // best of group s replaces the r-th worst of group s + 1 (mod S) when
      // strictly cheaper, all from the pre-migration state
      if (S > 1 && a.mig_interval > 0 && G > 1u && (G - 1u) % (uint32_t)a.mig_interval == 0u) {
        const int m = a.mig_count > 0 ? a.mig_count : max(1, NPs / 8), k = S * m;
        if (i < NP) {  // rank within the member's group, ties by index
          const int base = (i / NPs) * NPs;
          int r = 0;
          for (int j = base; j < base + NPs; ++j) r += (cost[j] < cost[i] || (cost[j] == cost[i] && j < i));
          byrank[base + r] = i;
        }
        __syncthreads();
        // copy each migrant into its target's spare row (sources are the
        // best m of a group, targets the worst m: disjoint as 2m <= NPs)
        for (int it = threadIdx.x; it < k * n; it += blockDim.x) {
          const int c = it / n, q = it - c * n, sg = c / m, r = c - sg * m;
          const int src = byrank[sg * NPs + r];
          const int dst = byrank[(sg + 1 == S ? 0 : sg + 1) * NPs + NPs - 1 - r];
          row(dst, cur[dst] ^ 1)[q] = row(src, cur[src])[q];
        }
        __syncthreads();
        int acc = 0;
        if (i < k) {
          const int sg = i / m, r = i - sg * m;
          const int src = byrank[sg * NPs + r];
          const int dst = byrank[(sg + 1 == S ? 0 : sg + 1) * NPs + NPs - 1 - r];
          const int32_t cs = cost[src];
          if (cs < cost[dst]) {
            cur[dst] ^= 1;
            cost[dst] = cs;
            acc = 1;
          }
        }
        if (acc && a.stats) atomicAdd(a.stats + 2, 1ull);
        __syncthreads();
      }
      if (i < NP) {
        const U4 ws = draw(a.seed, (uint32_t)t, G, (uint32_t)i, P_SELECT, 0);
        // binary tournaments within the member's sub-island
        const uint32_t us = (uint32_t)NPs;
        const int gb = (i / NPs) * NPs;
        const int p1 = better(cost, gb + (int)(ws.x % us), gb + (int)(ws.y % us));
        const int p2 = better(cost, gb + (int)(ws.z % us), gb + (int)(ws.w % us));
        const uint8_t* A = row(p1, cur[p1]);
        const uint8_t* B = row(p2, cur[p2]);
        uint8_t* c = row(i, cur[i] ^ 1);
        const U4 wo = draw(a.seed, (uint32_t)t, G, (uint32_t)i, P_OX, 0);
        if (u01(wo.x) < a.p_cross) {
          const int c1 = (int)(wo.y % (uint32_t)n), c2 = (int)(wo.z % (uint32_t)n);
          const int lo = c1 < c2 ? c1 : c2, hi = c1 < c2 ? c2 : c1;
          for (int q = 0; q < UW; ++q) used[q * P] = 0u;
          for (int k = lo; k <= hi; ++k) {
            const uint8_t gene = A[k];
            c[k] = gene;
            used[(gene >> 5) * P] |= 1u << (gene & 31);
          }
          int pos = hi + 1 == n ? 0 : hi + 1;
          int src = pos;
          for (int k = 0; k < n; ++k) {
            const uint8_t gene = B[src];
            src = src + 1 == n ? 0 : src + 1;
            const bool fresh = !((used[(gene >> 5) * P] >> (gene & 31)) & 1u);
            if (fresh) c[pos] = gene;
            pos = fresh ? (pos + 1 == n ? 0 : pos + 1) : pos;
          }
        } else {
          for (int k = 0; k < n; ++k) c[k] = A[k];
        }
        const U4 wm = draw(a.seed, (uint32_t)t, G, (uint32_t)i, P_MUTATE, 0);
        if (u01(wm.x) < a.p_swap) {
          const int s1 = (int)(wm.y % (uint32_t)n), s2 = (int)(wm.z % (uint32_t)n);
          const uint8_t tmp = c[s1];
          c[s1] = c[s2];
          c[s2] = tmp;
        }
        if (u01(wm.w) < a.p_2opt) {
          const U4 wr = draw(a.seed, (uint32_t)t, G, (uint32_t)i, P_MUTATE, 1);
          const int s1 = (int)(wr.x % (uint32_t)n), s2 = (int)(wr.y % (uint32_t)n);
          int lo = s1 < s2 ? s1 : s2, hi = s1 < s2 ? s2 : s1;
          while (lo < hi) {
            const uint8_t tmp = c[lo];
            c[lo] = c[hi];
            c[hi] = tmp;
            ++lo;
            --hi;
          }
        }
        kcost[i] = split_linear(n, node, d.capacity, c, rA, rQ, P, R);
      }
      __syncthreads();  // all children built from the old island
      if (i < NP && kcost[i] <= cost[i]) {
        cur[i] ^= 1;
        cost[i] = kcost[i];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      a.gen[t] = gen0 + (uint32_t)a.gens;
      if (a.stats) atomicAdd(a.stats + 0, (unsigned long long)NP * (unsigned long long)a.gens);
    }
    if (a.transfer_export && a.elites_out) {
      rank_members(cost, NP, byrank);
      int k = (int)(a.transfer_rate * (float)NP + 0.5f);
      k = k < 1 ? 1 : (k > NP ? NP : k);
      uint8_t* el = a.elites_out + d.elite_off;
      for (int it = threadIdx.x; it < k * n; it += blockDim.x) {
        const int c = it / n, q = it - c * n;
        const int m = byrank[c];
        el[it] = row(m, cur[m])[q];
      }
    }
  }
  __syncthreads();
  for (int it = threadIdx.x; it < NP * n; it += blockDim.x) {
    const int m = it / n, q = it - m * n;
    gpop[it] = row(m, cur[m])[q];
  }
  for (int it = threadIdx.x; it < NP; it += blockDim.x) a.cost[d.cost_off + it] = cost[it];
}

// Costs of caller-given tours of one instance: thread = tour.
template <int QB>
__global__ void __launch_bounds__(256) cvrp_eval_kernel(const Args a, int inst, int count,
                                                        const uint8_t* perms, int32_t* costs) {
  extern __shared__ __align__(16) unsigned char smem[];
  const InstDev d = a.inst[inst];
  const int n = d.n, P = blockDim.x;
  const Layout L = eval_layout(n, P, a.ring, QB);
  if (n < 1 || n > kMaxN || L.total > a.smem_bytes) {
    if (threadIdx.x == 0) report(a.err, 2);
    return;
  }
  int4* node = (int4*)(smem + L.node);
  int32_t* rA = (int32_t*)(smem + L.ringA) + threadIdx.x;
  const QRing<QB> rQ(smem + L.ringQ, threadIdx.x, P);
  load_instance(a, d, node);
  __syncthreads();
  const int k = blockIdx.x * P + threadIdx.x;
  if (k < count)
    costs[k] = split_linear(n, node, d.capacity, perms + (size_t)k * n, rA, rQ, P, a.ring);
}

// Best member of every instance.
__global__ void cvrp_best_kernel(const InstDev* inst, int n_inst, int NP, const int32_t* cost,
                                 int32_t* best_idx, int32_t* best_cost) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_inst) return;
  const InstDev d = inst[t];
  int bi = 0;
  for (int i = 1; i < NP; ++i)
    if (cost[d.cost_off + i] < cost[d.cost_off + bi]) bi = i;
  best_idx[t] = bi;
  best_cost[t] = cost[d.cost_off + bi];
}

}  // namespace cvrp
}  // namespace emt

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

struct HostInst {
  int n = 0, capacity = 0;
  int lmax = 0;  // most customers one route can serve (smallest demands first)
  std::vector<int32_t> x, y, demand;
  std::vector<int32_t> d0;  // distance of every node to the depot
};

int route_bound(const HostInst& hi) {
  std::vector<int32_t> q(hi.demand.begin() + 1, hi.demand.end());
  std::sort(q.begin(), q.end());
  int64_t load = 0;
  int k = 0;
  while (k < (int)q.size() && load + q[k] <= hi.capacity) load += q[k++];
  return k;
}

// Per-handle kernel shape: deque slots (one more than the longest route,
// rounded up to a multiple of 4), bytes of a stored demand prefix (the
// smallest with 2 * capacity below its range), crossover bitmap words.
struct Shape {
  int ring = 4, qb = 1, uw = 1;
};

Shape shape_of(const std::vector<HostInst>& a, const std::vector<HostInst>& b = {}) {
  int lmax = 0, cap = 0, nmax = 0;
  for (const std::vector<HostInst>* set : {&a, &b})
    for (const HostInst& hi : *set) {
      lmax = std::max(lmax, hi.lmax);
      cap = std::max(cap, hi.capacity);
      nmax = std::max(nmax, hi.n);
    }
  Shape sh;
  sh.ring = std::max(4, (lmax + 1 + 3) / 4 * 4);
  sh.qb = 2 * cap <= 0xFF ? 1 : (2 * cap <= 0xFFFF ? 2 : 4);
  sh.uw = (nmax >> 5) + 1;
  return sh;
}

size_t epoch_smem(int n, int P, const Shape& sh) {
  return emt::cvrp::layout(n, P, sh.ring, sh.qb, sh.uw).total;
}

int block_threads(int pop) { return ((pop + 31) / 32) * 32; }

template <typename T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  ~Buf() { release(); }
  cudaError_t ensure(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (!count) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * count);
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace

struct emt_cvrp_handle {
  emt_cvrp_config cfg{};
  std::vector<HostInst> inst;
  std::vector<emt::cvrp::InstDev> table;
  bool uploaded = false, initialized = false;
  uint32_t gdone = 0;
  int parity = 0;
  Shape shape;
  int eval_threads = 32;
  size_t smem = 0, eval_smem = 0;
  std::string err;
  cudaStream_t stream = nullptr;
  Buf<emt::cvrp::InstDev> d_inst;
  Buf<int4> d_node;
  Buf<int32_t> d_cost, d_err, d_best_idx, d_best_cost;
  Buf<uint8_t> d_pop, d_elites[2];
  Buf<uint32_t> d_gen;
  Buf<unsigned long long> d_stats;

  int fail(int code, const std::string& m) {
    err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? EMT_ERR_OUT_OF_MEMORY : EMT_ERR_CUDA;
  }
};

namespace {

int cvrp_upload(emt_cvrp_handle* h) {
  if (h->uploaded) return EMT_OK;
  const int T = (int)h->inst.size();
  if (!T) return h->fail(EMT_ERR_STATE, "no instances");
  const int NP = h->cfg.pop;
  h->table.resize(T);
  int64_t nodes = 0, pop = 0, el = 0;
  int32_t cost = 0;
  size_t smem = 0;
  const Shape sh = shape_of(h->inst);
  const int P = block_threads(NP);
  for (int t = 0; t < T; ++t) {
    const HostInst& hi = h->inst[t];
    emt::cvrp::InstDev& d = h->table[t];
    d.n = hi.n;
    d.capacity = hi.capacity;
    d.node_off = nodes;
    nodes += hi.n + 1;
    d.pop_off = pop;
    pop += (int64_t)NP * hi.n;
    d.cost_off = cost;
    cost += NP;
    d.pad = 0;
    d.elite_off = el;
    el += (int64_t)NP * hi.n;
    smem = std::max(smem, epoch_smem(hi.n, P, sh));
  }
  h->smem = smem;
  h->shape = sh;
  // evaluation block: the most threads (128, 64, 32) whose rings fit; 32
  // always does, as the epoch layout of the same rings is larger
  int smax = 0;
  cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->cfg.device);
  for (int pe = 128; pe >= 32; pe >>= 1) {
    size_t es = 0;
    for (const HostInst& hi : h->inst)
      es = std::max(es, emt::cvrp::eval_layout(hi.n, pe, sh.ring, sh.qb).total);
    h->eval_threads = pe;
    h->eval_smem = es;
    if (es <= (size_t)smax) break;
  }
  std::vector<int4> hn((size_t)nodes);
  for (int t = 0; t < T; ++t) {
    const HostInst& hi = h->inst[t];
    for (int i = 0; i <= hi.n; ++i)
      hn[h->table[t].node_off + i] = make_int4(hi.x[i], hi.y[i], hi.d0[i], hi.demand[i]);
  }
  cudaError_t e;
  if ((e = cudaSetDevice(h->cfg.device)) != cudaSuccess) return h->cuda_fail(e, "cudaSetDevice");
  if ((e = h->d_inst.ensure(T)) || (e = h->d_node.ensure(hn.size())) ||
      (e = h->d_pop.ensure((size_t)pop)) || (e = h->d_cost.ensure((size_t)cost)) ||
      (e = h->d_gen.ensure(T)) || (e = h->d_stats.ensure(3)) || (e = h->d_err.ensure(1)) ||
      (e = h->d_best_idx.ensure(T)) || (e = h->d_best_cost.ensure(T)))
    return h->cuda_fail(e, "cudaMalloc");
  if (h->cfg.transfer_interval > 0 && T > 1)
    for (int b = 0; b < 2; ++b)
      if ((e = h->d_elites[b].ensure((size_t)el))) return h->cuda_fail(e, "cudaMalloc");
  if ((e = cudaMemcpy(h->d_inst.p, h->table.data(), sizeof(emt::cvrp::InstDev) * T, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(h->d_node.p, hn.data(), sizeof(int4) * hn.size(), cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(h->d_gen.p, 0, sizeof(uint32_t) * T)) ||
      (e = cudaMemset(h->d_stats.p, 0, sizeof(unsigned long long) * 3)) ||
      (e = cudaMemset(h->d_err.p, 0, sizeof(int32_t))))
    return h->cuda_fail(e, "upload");
  // the copies and memsets above run on the legacy default stream, which a
  // non-blocking caller stream does not wait for
  if ((e = cudaStreamSynchronize(nullptr)) != cudaSuccess) return h->cuda_fail(e, "upload");
  h->uploaded = true;
  h->initialized = false;
  return EMT_OK;
}

emt::cvrp::Args cvrp_args(emt_cvrp_handle* h, int mode) {
  emt::cvrp::Args a{};
  a.inst = h->d_inst.p;
  a.n_inst = (int32_t)h->inst.size();
  a.NP = h->cfg.pop;
  a.mode = mode;
  a.ring = h->shape.ring;
  a.used_words = h->shape.uw;
  a.node = h->d_node.p;
  a.pop = h->d_pop.p;
  a.cost = h->d_cost.p;
  a.gen = h->d_gen.p;
  a.seed = h->cfg.seed;
  a.p_cross = h->cfg.p_cross;
  a.p_swap = h->cfg.p_swap;
  a.p_2opt = h->cfg.p_2opt;
  a.transfer_rate = h->cfg.transfer_rate;
  a.stats = h->d_stats.p;
  a.err = h->d_err.p;
  a.smem_bytes = h->smem;
  a.subislands = h->cfg.subislands > 1 ? h->cfg.subislands : 1;
  a.mig_interval = h->cfg.migration_interval;
  a.mig_count = h->cfg.migration_count;
  return a;
}

int cvrp_launch(emt_cvrp_handle* h, const emt::cvrp::Args& a, void* stream) {
  auto kern = h->shape.qb == 1 ? emt::cvrp::cvrp_epoch_kernel<1>
             : h->shape.qb == 2 ? emt::cvrp::cvrp_epoch_kernel<2> : emt::cvrp::cvrp_epoch_kernel<4>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->smem);
  if (e != cudaSuccess) return h->cuda_fail(e, "cudaFuncSetAttribute");
  kern<<<(int)h->inst.size(), block_threads(h->cfg.pop), h->smem, (cudaStream_t)stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "cvrp launch");
  return EMT_OK;
}

}  // namespace

extern "C" {

void emt_cvrp_config_default(emt_cvrp_config* c) {
  if (!c) return;
  std::memset(c, 0, sizeof(*c));
  c->pop = 128;
  c->p_cross = 0.9f;
  c->p_swap = 0.2f;
  c->p_2opt = 0.2f;
  c->transfer_interval = 0;
  c->transfer_rate = 0.1f;
  c->seed = 1;
  c->device = 0;
}

int emt_cvrp_create(const emt_cvrp_config* cfg, emt_cvrp_handle_t** out) {
  if (!cfg || !out) return EMT_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->pop < 2 || cfg->pop > 256 || !(cfg->p_cross >= 0.f && cfg->p_cross <= 1.f) ||
      !(cfg->p_swap >= 0.f && cfg->p_swap <= 1.f) || !(cfg->p_2opt >= 0.f && cfg->p_2opt <= 1.f) ||
      cfg->transfer_interval < 0 || !(cfg->transfer_rate > 0.f && cfg->transfer_rate <= 1.f))
    return EMT_ERR_INVALID_ARG;
  // sub-islands: NP splits evenly into groups of at least 4, each sending at
  // most half of its members
  const int S = cfg->subislands > 1 ? cfg->subislands : 1;
  if (cfg->subislands < 0 || cfg->migration_interval < 0 || cfg->migration_count < 0 ||
      cfg->pop % S != 0 || (S > 1 && cfg->pop / S < 4) ||
      2 * (cfg->migration_count > 0 ? cfg->migration_count : std::max(1, cfg->pop / S / 8)) >
          cfg->pop / S)
    return EMT_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return EMT_ERR_CUDA;
  if (cfg->device < 0 || cfg->device >= ndev) return EMT_ERR_INVALID_ARG;
  emt_cvrp_handle* h = new (std::nothrow) emt_cvrp_handle();
  if (!h) return EMT_ERR_OUT_OF_MEMORY;
  h->cfg = *cfg;
  *out = h;
  return EMT_OK;
}

static int add_instances_impl(emt_cvrp_handle_t* h, int32_t n, const emt_cvrp_instance* in) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (n < 0 || (n > 0 && !in)) return h->fail(EMT_ERR_INVALID_ARG, "bad instance array");
  int smax = 0;
  cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->cfg.device);
  std::vector<HostInst> add;
  for (int k = 0; k < n; ++k) {
    const emt_cvrp_instance& d = in[k];
    const uint32_t id = (uint32_t)(h->inst.size() + add.size());
    if (d.customers < 1 || d.customers > EMT_CVRP_MAX_CUSTOMERS)
      return h->fail(EMT_ERR_INVALID_ARG, "instance " + std::to_string(k) + ": customers out of range");
    // demand prefix sums stay below 2^31: n * capacity <= 255 * 2^23
    if (d.capacity < 1 || d.capacity > (1 << 23))
      return h->fail(EMT_ERR_INVALID_ARG, "instance " + std::to_string(k) + ": capacity outside [1, 2^23]");
    HostInst hi;
    hi.n = d.customers;
    hi.capacity = d.capacity;
    const int W = hi.n + 1;
    hi.x.resize(W);
    hi.y.resize(W);
    hi.demand.resize(W);
    if (d.x && d.y && d.demand) {
      for (int i = 0; i < W; ++i) {
        hi.x[i] = d.x[i];
        hi.y[i] = d.y[i];
        hi.demand[i] = i == 0 ? 0 : d.demand[i];
        if (d.x[i] < 0 || d.y[i] < 0 || d.x[i] > 40000 || d.y[i] > 40000 || (i > 0 && d.demand[i] < 0))
          return h->fail(EMT_ERR_INVALID_ARG, "instance " + std::to_string(k) + ": coordinates outside [0, 40000] or negative demand");
      }
    } else {
      for (int i = 0; i < W; ++i) {
        const emt::U4 w = emt::draw(h->cfg.seed, id, 0, (uint32_t)i, emt::cvrp::P_NODE, 0);
        hi.x[i] = (int32_t)(w.x % 1000u);
        hi.y[i] = (int32_t)(w.y % 1000u);
        hi.demand[i] = i == 0 ? 0 : (int32_t)(1u + w.z % 10u);
      }
    }
    for (int i = 1; i < W; ++i)
      if (hi.demand[i] > hi.capacity)
        return h->fail(EMT_ERR_INVALID_ARG, "instance " + std::to_string(k) + ": a demand exceeds the capacity");
    hi.lmax = route_bound(hi);
    hi.d0.resize(W);
    for (int i = 0; i < W; ++i)
      hi.d0[i] = (int32_t)emt::cvrp::round_dist(hi.x[0], hi.y[0], hi.x[i], hi.y[i]);
    add.push_back(std::move(hi));
  }
  // the deque ring is sized for the handle's longest route, so recheck every island
  const int P = block_threads(h->cfg.pop);
  const Shape sh = shape_of(h->inst, add);
  for (const std::vector<HostInst>* set : {&h->inst, &add})
    for (const HostInst& hi : *set)
      if ((size_t)smax < epoch_smem(hi.n, P, sh))
        return h->fail(EMT_ERR_UNSUPPORTED, "an island of " + std::to_string(hi.n) +
                                                " customers does not fit in shared memory");
  for (auto& a : add) h->inst.push_back(std::move(a));
  h->uploaded = false;
  h->initialized = false;
  return EMT_OK;
}

// Host allocations that grow with the handle fail as EMT_ERR_OUT_OF_MEMORY
// instead of unwinding through the C ABI.
int emt_cvrp_add_instances(emt_cvrp_handle_t* h, int32_t n, const emt_cvrp_instance* in) {
  try {
    return add_instances_impl(h, n, in);
  } catch (const std::bad_alloc&) {
    return h ? h->fail(EMT_ERR_OUT_OF_MEMORY, "host memory") : EMT_ERR_OUT_OF_MEMORY;
  }
}

static int cvrp_reset_impl(emt_cvrp_handle_t* h, void* stream) {
  if (!h) return EMT_ERR_INVALID_ARG;
  int rc = cvrp_upload(h);
  if (rc) return rc;
  h->stream = (cudaStream_t)stream;
  rc = cvrp_launch(h, cvrp_args(h, 1), stream);
  if (rc) return rc;
  h->initialized = true;
  h->gdone = 0;
  h->parity = 0;
  return EMT_OK;
}

int emt_cvrp_reset(emt_cvrp_handle_t* h, void* stream) {
  try {
    return cvrp_reset_impl(h, stream);
  } catch (const std::bad_alloc&) {
    return h ? h->fail(EMT_ERR_OUT_OF_MEMORY, "host memory") : EMT_ERR_OUT_OF_MEMORY;
  }
}

int emt_cvrp_run(emt_cvrp_handle_t* h, int32_t generations, void* stream) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (generations < 0) return h->fail(EMT_ERR_INVALID_ARG, "negative generation count");
  if (!h->initialized) {
    int rc = emt_cvrp_reset(h, stream);
    if (rc) return rc;
  }
  h->stream = (cudaStream_t)stream;
  const int T = (int)h->inst.size();
  const int interval = (h->cfg.transfer_interval > 0 && T > 1) ? h->cfg.transfer_interval : 0;
  int left = generations;
  while (left > 0) {
    int g = left;
    bool imp = false, exp = false;
    if (interval) {
      imp = h->gdone > 0 && h->gdone % (uint32_t)interval == 0;
      g = std::min(left, interval - (int)(h->gdone % (uint32_t)interval));
      exp = (h->gdone + (uint32_t)g) % (uint32_t)interval == 0;
    }
    emt::cvrp::Args a = cvrp_args(h, 0);
    a.gens = g;
    if (interval) {
      a.transfer_import = imp ? 1 : 0;
      a.transfer_export = exp ? 1 : 0;
      a.elites_in = h->d_elites[h->parity ^ 1].p;
      a.elites_out = h->d_elites[h->parity].p;
    }
    int rc = cvrp_launch(h, a, stream);
    if (rc) return rc;
    if (interval && exp) h->parity ^= 1;
    h->gdone += (uint32_t)g;
    left -= g;
  }
  return EMT_OK;
}

int emt_cvrp_sync(emt_cvrp_handle_t* h) {
  if (!h) return EMT_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "stream synchronize");
  if (h->d_err.p) {
    int32_t code = 0;
    e = cudaMemcpy(&code, h->d_err.p, sizeof(code), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "error word");
    if (code) {
      cudaMemset(h->d_err.p, 0, sizeof(int32_t));
      cudaStreamSynchronize(nullptr);  // cleared before the next launch on any stream
      return h->fail(EMT_ERR_DEVICE_CHECK, "device check " + std::to_string(code));
    }
  }
  return EMT_OK;
}

int emt_cvrp_get_population(emt_cvrp_handle_t* h, int32_t inst, uint8_t* perms, int32_t* costs) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (inst < 0 || inst >= (int32_t)h->inst.size()) return h->fail(EMT_ERR_INVALID_ARG, "instance index");
  if (!h->initialized) {
    int rc = emt_cvrp_reset(h, h->stream);
    if (rc) return rc;
  }
  int rc = emt_cvrp_sync(h);
  if (rc) return rc;
  const emt::cvrp::InstDev& d = h->table[inst];
  cudaError_t e = cudaSuccess;
  if (perms) e = cudaMemcpy(perms, h->d_pop.p + d.pop_off, (size_t)h->cfg.pop * d.n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && costs)
    e = cudaMemcpy(costs, h->d_cost.p + d.cost_off, sizeof(int32_t) * h->cfg.pop, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return h->cuda_fail(e, "copy population");
  return EMT_OK;
}

int emt_cvrp_get_best_all(emt_cvrp_handle_t* h, int32_t* costs) {
  if (!h || !costs) return EMT_ERR_INVALID_ARG;
  if (!h->initialized) {
    int rc = emt_cvrp_reset(h, h->stream);
    if (rc) return rc;
  }
  const int T = (int)h->inst.size();
  emt::cvrp::cvrp_best_kernel<<<(T + 127) / 128, 128, 0, h->stream>>>(
      h->d_inst.p, T, h->cfg.pop, h->d_cost.p, h->d_best_idx.p, h->d_best_cost.p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return h->cuda_fail(e, "best launch");
  e = cudaMemcpyAsync(costs, h->d_best_cost.p, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) return h->cuda_fail(e, "copy best");
  return emt_cvrp_sync(h);
}

int emt_cvrp_get_instance(emt_cvrp_handle_t* h, int32_t inst, int32_t* x, int32_t* y,
                          int32_t* demand, int32_t* dist) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (inst < 0 || inst >= (int32_t)h->inst.size()) return h->fail(EMT_ERR_INVALID_ARG, "instance index");
  const HostInst& hi = h->inst[inst];
  const int W = hi.n + 1;
  if (x) std::memcpy(x, hi.x.data(), sizeof(int32_t) * W);
  if (y) std::memcpy(y, hi.y.data(), sizeof(int32_t) * W);
  if (demand) std::memcpy(demand, hi.demand.data(), sizeof(int32_t) * W);
  if (dist)
    for (int i = 0; i < W; ++i)
      for (int j = 0; j < W; ++j)
        dist[(size_t)i * W + j] = (int32_t)emt::cvrp::round_dist(hi.x[i], hi.y[i], hi.x[j], hi.y[j]);
  return EMT_OK;
}

int emt_cvrp_evaluate(emt_cvrp_handle_t* h, int32_t inst, int32_t count, const uint8_t* perms,
                      int32_t* costs) {
  if (!h) return EMT_ERR_INVALID_ARG;
  if (inst < 0 || inst >= (int32_t)h->inst.size()) return h->fail(EMT_ERR_INVALID_ARG, "instance index");
  if (count < 0 || (count > 0 && (!perms || !costs))) return h->fail(EMT_ERR_INVALID_ARG, "bad tour array");
  if (count == 0) return EMT_OK;
  const int n = h->inst[inst].n;
  std::vector<uint8_t> seen((size_t)n + 1);
  for (int32_t k = 0; k < count; ++k) {
    std::fill(seen.begin(), seen.end(), 0);
    for (int q = 0; q < n; ++q) {
      const uint8_t c = perms[(size_t)k * n + q];
      if (c < 1 || c > n || seen[c])
        return h->fail(EMT_ERR_INVALID_ARG, "tour " + std::to_string(k) + " is not a permutation of 1..n");
      seen[c] = 1;
    }
  }
  int rc = cvrp_upload(h);
  if (rc) return rc;
  rc = emt_cvrp_sync(h);
  if (rc) return rc;
  uint8_t* dp = nullptr;
  int32_t* dc = nullptr;
  cudaError_t e = cudaMalloc((void**)&dp, (size_t)count * n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dc, sizeof(int32_t) * count);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dp, perms, (size_t)count * n, cudaMemcpyHostToDevice, h->stream);
  auto kern = h->shape.qb == 1 ? emt::cvrp::cvrp_eval_kernel<1>
             : h->shape.qb == 2 ? emt::cvrp::cvrp_eval_kernel<2> : emt::cvrp::cvrp_eval_kernel<4>;
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->eval_smem);
  if (e == cudaSuccess) {
    emt::cvrp::Args a = cvrp_args(h, 0);
    a.smem_bytes = h->eval_smem;
    const int pe = h->eval_threads;
    kern<<<(count + pe - 1) / pe, pe, h->eval_smem, h->stream>>>(a, inst, count, dp, dc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(costs, dc, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dp);
  cudaFree(dc);
  if (e != cudaSuccess) return h->cuda_fail(e, "evaluate");
  return emt_cvrp_sync(h);
}

int emt_cvrp_get_stats(emt_cvrp_handle_t* h, emt_stats* out) {
  if (!h || !out) return EMT_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  out->n_tasks = (int32_t)h->inst.size();
  if (h->d_stats.p) {
    int rc = emt_cvrp_sync(h);
    if (rc) return rc;
    unsigned long long s[3];
    cudaError_t e = cudaMemcpy(s, h->d_stats.p, sizeof(s), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "copy stats");
    out->evaluations = s[0];
    out->transfers_accepted = s[1];
    out->migrations_accepted = s[2];
    out->generations = h->initialized ? (uint64_t)h->gdone * h->inst.size() : 0;
  }
  return EMT_OK;
}

const char* emt_cvrp_last_error(const emt_cvrp_handle_t* h) { return h ? h->err.c_str() : "null handle"; }

void emt_cvrp_destroy(emt_cvrp_handle_t* h) {
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  h->d_inst.release();
  h->d_node.release();
  h->d_cost.release();
  h->d_err.release();
  h->d_best_idx.release();
  h->d_best_cost.release();
  h->d_pop.release();
  h->d_elites[0].release();
  h->d_elites[1].release();
  h->d_gen.release();
  h->d_stats.release();
  delete h;
}

}  // extern "C"
