/*
 * emt_oracle.h -- CPU ORACLE for the evolutionary-multitasking hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls
 * this code; tests/, the smoke check and the CPU-baseline leg of bench.py use
 * it as the checker and as the timed CPU restatement of the algorithm.
 *
 * It restates, in plain C, the reference's per-task generation step:
 *   - benchmark functions            proposed model/SG-EMTF.cu:898-1111
 *                                    (Griewank product: SG-EMTF_DE.cu:989)
 *   - box table                      SG-EMTF.cu:197-214
 *   - Weierstrass offset             SG-EMTF.cu:354-361
 *   - DE mutation / crossover        SG-EMTF_DE.cu:547-600, 474-495
 *   - SBX crossover, parent choice   SG-EMTF.cu:711-749, 772-831
 *   - polynomial mutation            SG-EMTF.cu:548-606
 *   - selection (ties to the child)  SG-EMTF_DE.cu:679-706
 *   - elite transfer                 SG-EMTF.cu:1514-1591
 * with the engine's own random stream (Philox4x32-10, Salmon et al., SC'11)
 * in place of the reference's time-seeded cuRAND XORWOW, so that a run can be
 * replayed bit for bit.
 *
 * Pinning.  The reference ships no test vectors.  The oracle is pinned by
 * (1) the Random123 known-answer vectors for Philox4x32-10, (2) analytic
 * optima of the seven functions, and (3) a statistical comparison with the
 * reference's own recorded GA trajectories (data process/ANO_Tnum/
 * data_record_T_ANO_100.txt, 18 runs x 100 tasks), regenerated by
 * tests/golden/make_reference_records.py.  Bit-level parity with the
 * reference's cuRAND stream and CUDA math is unpinned by construction: the
 * reference reseeds from time(0) (SG-EMTF.cu:376).
 *
 * Build: make -C oracle   (gcc, -ffp-contract=off so that a*b+c is never
 * fused behind our back; every intended fusion is an explicit fmaf()).
 */
#ifndef EMT_ORACLE_H
#define EMT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- function ids (same order as the engine's emt_function) ---- */
enum { ORC_SPHERE = 0, ORC_RASTRIGIN, ORC_ACKLEY, ORC_GRIEWANK, ORC_ROSENBROCK,
       ORC_SCHWEFEL, ORC_WEIERSTRASS, ORC_NFUNC };

enum { ORC_DE_RAND1 = 0, ORC_DE_CURRENT1 = 1, ORC_GA = 2 };

#define ORC_FLAG_REF_GRIEWANK_NO_PRODUCT 0x1u
#define ORC_FLAG_REF_WEIERSTRASS_CONST 0x2u
#define ORC_FLAG_REF_ACKLEY_E 0x4u
#define ORC_FLAG_REF_BOXES 0x8u
#define ORC_FLAG_NO_RECHECK 0x10u
#define ORC_FLAG_RIGOROUS_WINDOW 0x20u

/* ---- Philox4x32-10 and the stream layout shared with the engine ----
 * key = (seed low 32 bits, seed high 32 bits)
 * ctr = (task, generation, member, purpose << 24 | block)               */
enum {
  ORC_P_POP_INIT = 1, ORC_P_SHIFT = 2, ORC_P_QR_NORMAL = 3, ORC_P_DE_INDEX = 4,
  ORC_P_DE_CR = 5, ORC_P_GA_PARENT = 6, ORC_P_GA_SBX = 7, ORC_P_GA_PM = 8,
  ORC_P_TRANSFER_PARTNER = 9, ORC_P_TRANSFER_MIX = 10,
  /* CVRP (emt_cvrp_oracle.c) */
  ORC_P_CVRP_NODE = 16,     /* gen 0, member = node, block 0 -> x, y, demand   */
  ORC_P_CVRP_POP_INIT = 17, /* gen 0, member i, block b -> Fisher-Yates words  */
  ORC_P_CVRP_SELECT = 18,   /* gen g, member i -> two binary tournaments       */
  ORC_P_CVRP_OX = 19,       /* gen g, member i -> (p_cross, cut1, cut2, -)     */
  ORC_P_CVRP_MUTATE = 20,   /* gen g, member i, block 0 -> (p_swap, s1, s2, p_2opt),
                               block 1 -> (r1, r2, -, -)                      */
  ORC_P_CVRP_PARTNER = 21   /* gen g, member 0 -> transfer partner            */
};

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_draw(uint64_t seed, uint32_t task, uint32_t gen, uint32_t member,
              uint32_t purpose, uint32_t block, uint32_t out[4]);
float orc_u01(uint32_t w); /* (w >> 8) * 2^-24, in [0, 1) */

/* ---- tasks ---- */
typedef struct orc_task {
  int fid, D, NP;
  float lo, hi;
  const float* Q; /* D*D row-major FP32; NULL = identity */
  const float* o; /* D */
  uint32_t flags;
  uint32_t id;    /* task index in the Philox counter */
} orc_task;

typedef struct orc_params {
  int algorithm;
  float F, CR, eta_c, p_c, eta_m, p_m;
  float transfer_mix; /* probability a candidate gene comes from the partner */
  uint64_t seed;
  double recheck_rel;
  uint32_t flags;
  int subislands;   /* sub-islands per island (1 = one island); operators draw
                       partners within the member's sub-island            */
  int mig_interval; /* generations between ring migrations (0 = none)     */
  int mig_count;    /* members each sub-island sends                      */
} orc_params;

int orc_box(int fid, int reference_boxes, float* lo, float* hi);
int orc_function_from_reference(int reference_type);
double orc_weierstrass_reference_offset(void); /* SG-EMTF.cu:354-361 */

void orc_gen_shift(uint64_t seed, uint32_t task, int D, float lo, float hi, float* o);
void orc_gen_population(uint64_t seed, uint32_t task, int NP, int D, float lo, float hi,
                        float* X);
void orc_gen_rotation(uint64_t seed, uint32_t task, int D, double* Q);

/* FP64 evaluation of one point.  z (optional) receives the rotated argument,
 * scale (optional) the sum of absolute sub-terms used in the error metric
 * |f - f64| / scale. */
double orc_eval64(const orc_task* t, const float* x, double* scale, double* z);
/* FP32 evaluation, same operation order as the engine's FP32 form (the CPU
 * baseline's arithmetic). */
float orc_eval32(const orc_task* t, const float* x, float* scale);
/* First-order bound on |f(z_fp32) - f(z_exact)| for Weierstrass, caused by
 * FP32 rounding of the rotation (see the engine's error model). */
double orc_weierstrass_rotation_bound(const orc_task* t, const float* x);

/* ---- one generation of one task ----
 * X: NP*D FP32 population (row-major), fit32/fit64: fitness of each member
 * (fit64 NaN = unknown).  gen: 1-based generation number.
 * mode 0: every selection decided in FP64 (ideal replay).
 * mode 1: FP32 fitness, FP64 re-check inside the window (the engine's rule).
 * accepted (optional, NP bytes) receives the selection mask.
 * Returns the number of FP64 re-checks.                                    */
int orc_generation(const orc_params* p, const orc_task* t, float* X, float* fit32,
                   double* fit64, uint32_t gen, int mode, uint8_t* accepted);
/* The trial vector of member i (bit-exact with the engine). */
void orc_trial(const orc_params* p, const orc_task* t, const float* X, uint32_t gen,
               int i, float* u);
float orc_powf(float x, float y); /* the engine's deterministic power */

/* Rank of every member by (fit32, index), ascending: rank[i] in [0, NP). */
void orc_rank(const float* fit32, int NP, int* rank);

/* Elite transfer into task t from partner p (elites: partner's top k rows,
 * k*Dp floats with row stride Dp).  gen: the generation number after which
 * the transfer happens.  Returns the number of members replaced. */
/* Ring migration between the sub-islands of one island (IslandMigration,
 * SG-EMTF.cu:1138-1218, generalised from two slots to a ring): ranks each
 * sub-island by fit32; the i-th best of sub-island s replaces the i-th worst
 * of s + 1 when strictly better (FP64 in mode 0), all from the
 * pre-migration state.  Runs before the trials of generation gen when
 * orc_migration_due(p, gen).  Returns the replacements. */
int orc_migration_due(const orc_params* p, uint32_t gen);
int orc_migration_count(const orc_params* p, int NP);
int orc_migrate(const orc_params* p, const orc_task* t, float* X, float* fit32, double* fit64,
                int mode);
int orc_transfer_partner(const orc_params* p, uint32_t t, uint32_t n_tasks, uint32_t gen);
int orc_transfer_in(const orc_params* p, const orc_task* t, const orc_task* partner,
                    const float* elites, int k, float* X, float* fit32, double* fit64,
                    uint32_t gen, int mode);

/* Multi-threaded CPU run (the timed CPU baseline): n tasks, each with its own
 * state, `gens` generations, mode as orc_generation.  Returns wall seconds. */
double orc_run_threads(const orc_params* p, const orc_task* tasks, int n, float** X,
                       float** fit32, double** fit64, uint32_t gen0, int gens, int mode,
                       int threads);

/* ---- CVRP (emt_cvrp_oracle.c) ---- */
typedef struct orc_cvrp_params {
  uint64_t seed;
  float p_cross, p_swap, p_2opt;
  /* sub-islands: groups per island (<= 1: one), migration interval, count */
  int subislands, mig_interval, mig_count;
} orc_cvrp_params;

uint32_t orc_cvrp_round_sqrt(uint64_t v);
void orc_cvrp_gen_instance(uint64_t seed, uint32_t inst, int n, int32_t* x, int32_t* y,
                           int32_t* demand);
void orc_cvrp_distances(int n, const int32_t* x, const int32_t* y, int32_t* dist);
int32_t orc_cvrp_split(int n, const int32_t* dist, const int32_t* demand, int32_t capacity,
                       const uint8_t* perm, int32_t* pred);
void orc_cvrp_child(const orc_cvrp_params* p, uint32_t inst, int n, int NP, const uint8_t* pop,
                    const int32_t* cost, uint32_t g, int i, uint8_t* child);
void orc_cvrp_init_population(uint64_t seed, uint32_t inst, int n, int NP, uint8_t* pop);
int orc_cvrp_generation(const orc_cvrp_params* p, uint32_t inst, int n, int NP,
                        const int32_t* dist, const int32_t* demand, int32_t capacity,
                        uint8_t* pop, int32_t* cost, uint32_t g);
void orc_cvrp_rank(const int32_t* cost, int NP, int* byrank);
/* Ring migration between the CVRP island's sub-islands before generation g
 * (when due): the r-th best of group s replaces the r-th worst of group
 * s + 1 (mod S) when strictly cheaper, all from the pre-migration state
 * (the reference's IslandMigration, SG-EMTF_cvrp.cu:965-1020).  Returns the
 * replacements. */
int orc_cvrp_migrate(const orc_cvrp_params* p, int n, int NP, uint8_t* pop, int32_t* cost,
                     uint32_t g);
int orc_cvrp_transfer_in(int n, int NP, const int32_t* dist, const int32_t* demand,
                         int32_t capacity, const uint8_t* elites, int k, uint8_t* pop,
                         int32_t* cost);

#ifdef __cplusplus
}
#endif
#endif
