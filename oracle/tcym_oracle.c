/*
 * ORACLE — test infrastructure, not product.
 *
 * FP64 CPU restatement of the real-time lattice Yang-Mills hot path of
 * markmace/TopologicalCYMSolver (leapfrog, Langevin, gradient flow, Gauss
 * restore, observables, clover E.B), in plain C with OpenMP over z as the
 * reference parallelises (DYNAMICS/Dynamics.cpp:106-136).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm load it,
 * to check or time against.  The CUDA product never links or calls it.
 *
 * Parity pin: this restatement is checked in tests/test_oracle_golden.py
 * against golden vectors produced by the reference's own sources compiled
 * here (oracle/ref_wrap.cpp, fixtures under tests/golden/, generator
 * tests/golden/make_golden.py).
 *
 * Exported symbols: orc_su2_* and orc_su3_* (see orc_lattice.inc), and
 * orc_philox4x32 / orc_normal_c for the RNG known-answer tests.
 */
#include <stdint.h>
#include <stdlib.h>

#include "orc_group.h"
#include "orc_philox.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846264338327950288
#endif

void orc_philox4x32(const uint32_t *ctr, const uint32_t *key, uint32_t *out) { orc_philox4x32_10(ctr, key, out); }
double orc_normal_c(uint64_t seed, uint32_t stream, uint64_t step, uint32_t site, uint32_t mu, uint32_t a) {
    return orc_normal(seed, stream, step, site, mu, a);
}

/* ---- SU(2) instantiation ---- */
#define PFX(name) orc_su2_##name
#define MAT double
#define NM 4
#define NA 3
#define G_MUL su2_mul
#define G_DAG su2_dag
#define G_IDENT su2_identity
#define G_PROJ su2_proj
#define G_RETR1M su2_retr_one_minus
#define G_IEXP su2_iexp
#define G_ADJ su2_adjoint
#define G_INVADJ su2_inverse_adjoint
#define G_UNORM su2_unitarity_norm
#define G_ILOG su2_ilog
#include "orc_lattice.inc"
#undef PFX
#undef MAT
#undef NM
#undef NA
#undef G_MUL
#undef G_DAG
#undef G_IDENT
#undef G_PROJ
#undef G_RETR1M
#undef G_IEXP
#undef G_ADJ
#undef G_INVADJ
#undef G_UNORM
#undef G_ILOG
#undef OFF

/* ---- SU(3) instantiation ---- */
#define PFX(name) orc_su3_##name
#define MAT cplx
#define NM 9
#define NA 8
#define G_MUL su3_mul
#define G_DAG su3_dag
#define G_IDENT su3_identity
#define G_PROJ su3_proj
#define G_RETR1M su3_retr_one_minus
#define G_IEXP su3_iexp
#define G_ADJ su3_adjoint
#define G_INVADJ su3_inverse_adjoint
#define G_UNORM su3_unitarity_norm
#define G_ILOG su3_ilog
#include "orc_lattice.inc"
