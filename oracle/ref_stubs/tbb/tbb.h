/* Minimal stand-in for the parts of Intel TBB that the reference's
 * base/cpu_prop.cc uses (TBB is not installed).  Test infrastructure only:
 * it lets the reference CPU propagator compile from its own source into
 * oracle/_ref.  parallel_for splits the range over std::thread workers when
 * ORACLE_REF_THREADS > 1 (set at run time), else runs it inline.  The
 * propagator loops it drives are element-wise, so the split does not change
 * any result. */
#pragma once
#include "blocked_range.h"
#include "parallel_for.h"
#include "parallel_reduce.h"
