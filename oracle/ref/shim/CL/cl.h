/* Stand-in for the OpenCL header: the reference harness compiles pbrt's CPU
 * classes only, which name a few cl_* scalar types in their declarations. */
#ifndef ORACLE_REF_SHIM_CL_H
#define ORACLE_REF_SHIM_CL_H
#include <stdint.h>
typedef float cl_float;
typedef uint32_t cl_uint;
typedef int32_t cl_int;
typedef uint8_t cl_uchar;
typedef int8_t cl_char;
typedef uint64_t cl_ulong;
typedef struct { float s[4]; } cl_float4;
#endif
