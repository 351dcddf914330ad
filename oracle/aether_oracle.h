/*
 * aether_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of the reference's algorithms for the fused
 * batched-expression path: Philox4x32-10 and its keying, the distribution
 * leaves, the per-sample expression semantics (one node at a time, in the
 * reference's evaluation order) and the compensated-sum primitives.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference legs may load this library, and only as the checker or the timed
 * CPU baseline. The product (aether_gb300) never links, loads or calls it.
 *
 * Parity pin: the Philox/keying functions are checked against the golden rows
 * of the reference's tests/random/golden_random.h (committed as fixtures under
 * tests/golden/), and the expression interpreter against outputs of the
 * reference headers compiled in AETHER_CPP_MODE by oracle/Makefile (target
 * `ref`), also committed as fixtures.
 */
#ifndef AETHER_ORACLE_H
#define AETHER_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Philox4x32-10 and keying (random/detail/Philox.h, Backend.h, Generator.h) ---- */
uint64_t orc_splitmix64(uint64_t x);
uint64_t orc_generator_key(uint64_t seed, uint64_t stream_id);
uint64_t orc_substream_key(uint64_t key, uint64_t k);
void orc_philox4x32_10(const uint32_t ctr[4], uint32_t key_x, uint32_t key_y, uint32_t out[4]);
uint64_t orc_random_bits64(uint64_t seed, uint32_t global, uint64_t counter);
double orc_uniform01_f64(uint64_t seed, uint32_t global, uint64_t counter);
float orc_uniform01_f32(uint64_t seed, uint32_t global, uint64_t counter);
double orc_normal_f64(uint64_t seed, uint32_t global, uint64_t counter);
float orc_normal_f32(uint64_t seed, uint32_t global, uint64_t counter);

/* ---- expression interpreter ---------------------------------------------------- */
typedef struct OrcOperand {
    const void* ptr;   /* plane 0 of the operand (host memory) */
    uint64_t pitch;    /* elements between component planes */
} OrcOperand;

typedef struct OrcArgs {
    uint64_t n;                 /* samples */
    uint32_t sample_offset;     /* global id of sample 0 */
    void* dst;                  /* output planes (host), dtype per `mode` */
    uint64_t dst_pitch;
    const OrcOperand* operands;
    uint32_t n_operands;
    const double* scalars;
    uint32_t n_scalars;
    const uint64_t* keys;
    uint32_t n_keys;
    double* reduce_out;         /* sum plans: (hi, comp) */
} OrcArgs;

/* mode: 0 = evaluate in the plan's own element type (the reference's semantics);
 *       1 = evaluate every node in double, write double (the FP64 oracle of an
 *           FP32 plan);
 *       2 = evaluate in long double, write double (error statistics). */
int orc_eval(const char* ir, int mode, const OrcArgs* args, int nthreads);
const char* orc_last_error(void);

/* ---- compensated sums (accum/atomic.h, accum/TwoSum.h) ---------------------------- */
void orc_pair_combine_f64(double ah, double ac, double bh, double bc, double* oh, double* oc);
void orc_neumaier_add_f64(double* hi, double* comp, double term);
void orc_reduce32_f64(const double* hi32, const double* comp32, double* oh, double* oc);
void orc_reduce32_f32(const float* hi32, const float* comp32, float* oh, float* oc);

/* ---- the reference's user loops for the benchmark workloads, OpenMP ---------------- *
 * Each is the `#pragma omp parallel for` over samples with `dst[i] = expr` that a
 * consumer of the reference writes; nthreads <= 0 uses every host thread. */
void orc_fill_uniform_f64(uint64_t key, double lo, double hi, int comps, uint64_t n, uint64_t pitch, double* out,
                          int nthreads);
void orc_fill_uniform_f32(uint64_t key, float lo, float hi, int comps, uint64_t n, uint64_t pitch, float* out,
                          int nthreads);
void orc_fill_normal_f64(uint64_t key, double mean, double sd, int comps, uint64_t n, uint64_t pitch, double* out,
                         uint32_t sample_offset, int nthreads);
/* d = a + b*c + sin(a)*exp((c*c)*(-1.0)), Array<double,3> */
void orc_cfg1_f64(const double* a, const double* b, const double* c, double* d, uint64_t n, uint64_t pitch,
                  int nthreads);
/* d = sqrt(a*a+b*b) * log1p(|c|) + rsqrt(1 + d0*d0), Array<double,3> */
void orc_cfg2a_f64(const double* a, const double* b, const double* c, const double* d0, double* d, uint64_t n,
                   uint64_t pitch, int nthreads);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
