/*
 * emt_cvrp_oracle.c -- CPU ORACLE for the CVRP multitask engine (test
 * infrastructure only; see emt_oracle.h for what may use it).
 *
 * The reference's CVRP variant (proposed model/SG-EMTF_cvrp.cu) is
 * unfinished: its crossover computes a repair and then sets every gene to 1
 * (:731-736), its distances are random asymmetric floats (:210-225) and its
 * capacity counts customers (:932-944).  Parity with it is therefore
 * unpinned; this oracle restates the published methods the engine
 * implements, in integer arithmetic only, so the device must match it bit
 * for bit:
 *   - instances: integer coordinates uniform on [0, 1000)^2, demands uniform
 *     in 1..10, depot 0 with demand 0; rounded Euclidean distances
 *     round(sqrt(dx^2 + dy^2)) computed with an integer square root;
 *   - giant-tour encoding (a permutation of customers 1..n) decoded by the
 *     split procedure of Prins (Computers & Operations Research 31, 2004):
 *     shortest path over capacity-feasible consecutive segments;
 *   - order crossover (Davis 1985), swap and 2-opt (segment reversal)
 *     mutation, binary tournaments, child i replaces member i when not worse
 *     (the reference's selection rule, SG-EMTF.cu:752-769);
 *   - elite transfer of whole permutations between instances with the same
 *     number of customers (knowledgeTransfer, SG-EMTF.cu:1514-1591).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "emt_oracle.h"

/* floor(sqrt(v)) exactly, by bisection on integers */
static uint32_t isqrt_u64(uint64_t v) {
  uint64_t lo = 0, hi = 1u << 21;  /* v < 2^42 */
  while (lo < hi) {
    uint64_t mid = (lo + hi + 1) >> 1;
    if (mid * mid <= v) lo = mid; else hi = mid - 1;
  }
  return (uint32_t)lo;
}

/* round(sqrt(v)): r = floor(sqrt(v)); sqrt(v) < r + 1/2 <=> v <= r^2 + r */
uint32_t orc_cvrp_round_sqrt(uint64_t v) {
  uint32_t r = isqrt_u64(v);
  return (v <= (uint64_t)r * r + r) ? r : r + 1u;
}

void orc_cvrp_gen_instance(uint64_t seed, uint32_t inst, int n, int32_t* x, int32_t* y,
                           int32_t* demand) {
  uint32_t w[4];
  for (int i = 0; i <= n; ++i) {
    orc_draw(seed, inst, 0, (uint32_t)i, ORC_P_CVRP_NODE, 0, w);
    x[i] = (int32_t)(w[0] % 1000u);
    y[i] = (int32_t)(w[1] % 1000u);
    demand[i] = i == 0 ? 0 : (int32_t)(1u + w[2] % 10u);
  }
}

void orc_cvrp_distances(int n, const int32_t* x, const int32_t* y, int32_t* dist) {
  for (int i = 0; i <= n; ++i)
    for (int j = 0; j <= n; ++j) {
      int64_t dx = x[i] - x[j], dy = y[i] - y[j];
      dist[i * (n + 1) + j] = (int32_t)orc_cvrp_round_sqrt((uint64_t)(dx * dx + dy * dy));
    }
}

/* Prins split: V[j] = min over feasible segments (i, j] of V[i] + route cost */
int32_t orc_cvrp_split(int n, const int32_t* dist, const int32_t* demand, int32_t capacity,
                       const uint8_t* perm, int32_t* pred) {
  const int W = n + 1;
  int32_t V[256];
  V[0] = 0;
  for (int j = 1; j <= n; ++j) V[j] = INT32_MAX;
  for (int i = 0; i < n; ++i) {
    if (V[i] == INT32_MAX) continue;
    int32_t load = 0, cost = 0;
    for (int j = i + 1; j <= n; ++j) {
      const int c = perm[j - 1];
      load += demand[c];
      if (load > capacity) break;
      if (j == i + 1) {
        cost = dist[c] + dist[c * W];
      } else {
        const int p = perm[j - 2];
        cost = cost - dist[p * W] + dist[p * W + c] + dist[c * W];
      }
      if (V[i] + cost < V[j]) {
        V[j] = V[i] + cost;
        if (pred) pred[j] = i;
      }
    }
  }
  return V[n];
}

static int better(const int32_t* cost, int a, int b) {
  return (cost[a] < cost[b] || (cost[a] == cost[b] && a <= b)) ? a : b;
}

int orc_cvrp_migrate(const orc_cvrp_params* p, int n, int NP, uint8_t* pop, int32_t* cost,
                     uint32_t g);

/* Child of member i in generation g (bit-exact with the device). */
void orc_cvrp_child(const orc_cvrp_params* p, uint32_t inst, int n, int NP, const uint8_t* pop,
                    const int32_t* cost, uint32_t g, int i, uint8_t* child) {
  uint32_t w[4], v[4], m[4], r[4];
  orc_draw(p->seed, inst, g, (uint32_t)i, ORC_P_CVRP_SELECT, 0, w);
  /* tournaments within the member's sub-island of NPs members */
  const int S = p->subislands > 1 ? p->subislands : 1, NPs = NP / S, base = (i / NPs) * NPs;
  const int p1 = better(cost, base + (int)(w[0] % (uint32_t)NPs), base + (int)(w[1] % (uint32_t)NPs));
  const int p2 = better(cost, base + (int)(w[2] % (uint32_t)NPs), base + (int)(w[3] % (uint32_t)NPs));
  const uint8_t* a = pop + (size_t)p1 * n;
  const uint8_t* b = pop + (size_t)p2 * n;
  orc_draw(p->seed, inst, g, (uint32_t)i, ORC_P_CVRP_OX, 0, v);
  if (orc_u01(v[0]) < p->p_cross) {
    int c1 = (int)(v[1] % (uint32_t)n), c2 = (int)(v[2] % (uint32_t)n);
    int lo = c1 < c2 ? c1 : c2, hi = c1 < c2 ? c2 : c1;
    uint8_t used[256];
    memset(used, 0, sizeof(used));
    for (int k = lo; k <= hi; ++k) {
      child[k] = a[k];
      used[a[k]] = 1;
    }
    int pos = (hi + 1) % n;
    for (int k = 0; k < n; ++k) {
      const uint8_t gene = b[(hi + 1 + k) % n];
      if (!used[gene]) {
        child[pos] = gene;
        pos = (pos + 1) % n;
      }
    }
  } else {
    memcpy(child, a, (size_t)n);
  }
  orc_draw(p->seed, inst, g, (uint32_t)i, ORC_P_CVRP_MUTATE, 0, m);
  if (orc_u01(m[0]) < p->p_swap) {
    const int s1 = (int)(m[1] % (uint32_t)n), s2 = (int)(m[2] % (uint32_t)n);
    const uint8_t t = child[s1];
    child[s1] = child[s2];
    child[s2] = t;
  }
  if (orc_u01(m[3]) < p->p_2opt) {
    orc_draw(p->seed, inst, g, (uint32_t)i, ORC_P_CVRP_MUTATE, 1, r);
    int s1 = (int)(r[0] % (uint32_t)n), s2 = (int)(r[1] % (uint32_t)n);
    int lo = s1 < s2 ? s1 : s2, hi = s1 < s2 ? s2 : s1;
    while (lo < hi) {
      const uint8_t t = child[lo];
      child[lo] = child[hi];
      child[hi] = t;
      ++lo;
      --hi;
    }
  }
}

void orc_cvrp_init_population(uint64_t seed, uint32_t inst, int n, int NP, uint8_t* pop) {
  uint32_t w[4];
  for (int i = 0; i < NP; ++i) {
    uint8_t* q = pop + (size_t)i * n;
    for (int k = 0; k < n; ++k) q[k] = (uint8_t)(k + 1);
    /* Fisher-Yates, one word per swap, words taken in order from blocks of 4 */
    for (int k = n - 1, t = 0; k > 0; --k, ++t) {
      if ((t & 3) == 0) orc_draw(seed, inst, 0, (uint32_t)i, ORC_P_CVRP_POP_INIT, (uint32_t)(t >> 2), w);
      const int j = (int)(w[t & 3] % (uint32_t)(k + 1));
      const uint8_t tmp = q[k];
      q[k] = q[j];
      q[j] = tmp;
    }
  }
}

int orc_cvrp_generation(const orc_cvrp_params* p, uint32_t inst, int n, int NP,
                        const int32_t* dist, const int32_t* demand, int32_t capacity,
                        uint8_t* pop, int32_t* cost, uint32_t g) {
  orc_cvrp_migrate(p, n, NP, pop, cost, g); /* when due, before the children */
  uint8_t* kids = (uint8_t*)malloc((size_t)NP * n);
  int32_t* kc = (int32_t*)malloc(sizeof(int32_t) * NP);
  int acc = 0;
  for (int i = 0; i < NP; ++i) {
    orc_cvrp_child(p, inst, n, NP, pop, cost, g, i, kids + (size_t)i * n);
    kc[i] = orc_cvrp_split(n, dist, demand, capacity, kids + (size_t)i * n, NULL);
  }
  for (int i = 0; i < NP; ++i)
    if (kc[i] <= cost[i]) {
      memcpy(pop + (size_t)i * n, kids + (size_t)i * n, (size_t)n);
      cost[i] = kc[i];
      ++acc;
    }
  free(kids);
  free(kc);
  return acc;
}

/* rank by (cost, index) */
void orc_cvrp_rank(const int32_t* cost, int NP, int* byrank) {
  for (int i = 0; i < NP; ++i) {
    int r = 0;
    for (int j = 0; j < NP; ++j) r += (cost[j] < cost[i] || (cost[j] == cost[i] && j < i)) ? 1 : 0;
    byrank[r] = i;
  }
}

/* Instance t receives the partner's k best permutations (elites, k*n bytes in
 * rank order); candidate c replaces t's member of rank NP-k+c if strictly
 * better.  Returns the number of replacements. */
int orc_cvrp_transfer_in(int n, int NP, const int32_t* dist, const int32_t* demand,
                         int32_t capacity, const uint8_t* elites, int k, uint8_t* pop,
                         int32_t* cost) {
  int byrank[256];
  orc_cvrp_rank(cost, NP, byrank);
  int target[256];
  for (int c = 0; c < k; ++c) target[c] = byrank[NP - k + c];
  int acc = 0;
  for (int c = 0; c < k; ++c) {
    const int32_t cc = orc_cvrp_split(n, dist, demand, capacity, elites + (size_t)c * n, NULL);
    const int m = target[c];
    if (cc < cost[m]) {
      memcpy(pop + (size_t)m * n, elites + (size_t)c * n, (size_t)n);
      cost[m] = cc;
      ++acc;
    }
  }
  return acc;
}

static int cvrp_mig_count(const orc_cvrp_params* p, int NPs) {
  if (p->mig_count > 0) return p->mig_count;
  const int m = NPs / 8;
  return m < 1 ? 1 : m;
}

int orc_cvrp_migrate(const orc_cvrp_params* p, int n, int NP, uint8_t* pop, int32_t* cost,
                     uint32_t g) {
  const int S = p->subislands > 1 ? p->subislands : 1;
  if (S < 2 || p->mig_interval <= 0 || g <= 1u || (g - 1u) % (uint32_t)p->mig_interval != 0u)
    return 0;
  const int NPs = NP / S, m = cvrp_mig_count(p, NPs), k = S * m;
  int* byrank = (int*)malloc(sizeof(int) * NP);
  for (int i = 0; i < NP; ++i) { /* rank within the member's sub-island */
    const int base = (i / NPs) * NPs;
    int r = 0;
    for (int j = base; j < base + NPs; ++j)
      if (cost[j] < cost[i] || (cost[j] == cost[i] && j < i)) ++r;
    byrank[base + r] = i;
  }
  uint8_t* C = (uint8_t*)malloc((size_t)k * n);
  int32_t* cc = (int32_t*)malloc(sizeof(int32_t) * k);
  int* target = (int*)malloc(sizeof(int) * k);
  for (int c = 0; c < k; ++c) {
    const int s = c / m, r = c - s * m, d = (s + 1) % S, src = byrank[s * NPs + r];
    memcpy(C + (size_t)c * n, pop + (size_t)src * n, (size_t)n);
    cc[c] = cost[src];
    target[c] = byrank[d * NPs + NPs - 1 - r];
  }
  int acc = 0;
  for (int c = 0; c < k; ++c)
    if (cc[c] < cost[target[c]]) {
      memcpy(pop + (size_t)target[c] * n, C + (size_t)c * n, (size_t)n);
      cost[target[c]] = cc[c];
      ++acc;
    }
  free(C);
  free(cc);
  free(target);
  free(byrank);
  return acc;
}
