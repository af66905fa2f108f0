// clshim_pre.h — included at global scope before a per-file namespace that
// holds clshim_body.h and one reference kernels/*.cl file.  Test
// infrastructure only (builds oracle/_ref from the reference sources).
#pragma once
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include <float.h>
#include <string.h>
#include "../../raccoongpurender_gb300/csrc/rgr_fmath.h"
#include "../rgr_oracle.h"

extern thread_local size_t rgr_cl_gid;
extern thread_local size_t rgr_cl_gsize;

#define __kernel
#define __global
#define __local
#define __constant const
#define __read_only
#define __write_only
