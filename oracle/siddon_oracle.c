/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.  Not part of the product: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and only
 * as the checker / CPU baseline.
 *
 * A plain-C (C99 + OpenMP) restatement of TomograPy's Siddon conic projector,
 * tomograpy/C_siddon.c.template, in double and float, with the reference's
 * four accumulate modes (pj, bpj, pjt, bpjt) and two obstacles (none, sun).
 * Parity is pinned against the reference itself: tests/golden/ holds outputs
 * of the reference's own compiled template (oracle/build_ref.py builds it,
 * tests/golden/make_golden.py runs it) and tests/test_oracle_golden.py checks
 * this file against them.
 *
 * Deliberate interface differences from the CPython module: headers arrive as
 * C structs (the reference reads them from .header dicts,
 * tomograpy/C_siddon.c.template:1051-1101), arrays as base pointer + element
 * strides, and the mask is passed in the data's own element type (the
 * reference reads its mask with the data's C type,
 * tomograpy/C_siddon.c.template:29-31,520).
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (see oracle/__init__.py).
 */
#include <math.h>
#include <omp.h>
#include <stddef.h>

#include "siddon_oracle.h"

#define ORACLE_INF 100000 /* tomograpy/C_siddon.c.template:17 */

#define CT double
#define SFX f64
#include "siddon_oracle_body.h"
#undef CT
#undef SFX

#define CT float
#define SFX f32
#include "siddon_oracle_body.h"
#undef CT
#undef SFX

int oracle_version(void) { return 1; }
