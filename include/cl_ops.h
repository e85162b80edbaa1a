/*
 * cl_ops on GB300 -- aggregate header (reference: src/cl_ops/cl_ops.h:34-48).
 */
#ifndef CL_OPS_H
#define CL_OPS_H

#include "clo_common.h"
#include "ccl_shim.h"
#include "clo_sort_abstract.h"
#include "clo_scan_abstract.h"
#include "clo_rng.h"
#include "clo_gb300.h"
#include "clo_serve.h"

#endif /* CL_OPS_H */
