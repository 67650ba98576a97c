/* ORACLE - test infrastructure only; see oracle.h. */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../parallel_tree_hmm_gb300/csrc/portable_math.h"

#define S double
#define SFX(name) name##_f64
#define XEXP(x, math) ((math) ? thmm_exp(x) : exp(x))
#define XLOG(x, math) ((math) ? thmm_log(x) : log(x))
#define XLOGREF(x) log(x)
#include "oracle_impl.h"
#undef S
#undef SFX
#undef XEXP
#undef XLOG
#undef XLOGREF

#define S float
#define SFX(name) name##_f32
#define XEXP(x, math) ((math) ? thmm_expf(x) : expf(x))
#define XLOG(x, math) ((math) ? thmm_logf(x) : logf(x))
#define XLOGREF(x) logf(x)
#include "oracle_impl.h"
#undef S
#undef SFX
#undef XEXP
#undef XLOG
#undef XLOGREF

float oracle_portable_expf(float x) { return thmm_expf(x); }
float oracle_portable_logf(float x) { return thmm_logf(x); }
double oracle_portable_exp(double x) { return thmm_exp(x); }
double oracle_portable_log(double x) { return thmm_log(x); }
