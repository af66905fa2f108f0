// Work-item ids for the reference kernels compiled by the shim (test infrastructure).
#include <stddef.h>
thread_local size_t rgr_cl_gid = 0;
thread_local size_t rgr_cl_gsize = 0;
