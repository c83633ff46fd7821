/* Shadows core/GPUparallel.h for the reference harness: the OpenCL wrapper
 * classes are declared but never defined or used by the CPU classes that the
 * harness links. */
#ifndef ORACLE_REF_SHIM_GPUPARALLEL_H
#define ORACLE_REF_SHIM_GPUPARALLEL_H
#include <CL/cl.h>
#include "core/parallel.h"
#include "core/error.h"
class OpenCL;
class OpenCLTask;
class OpenCLQueue;
#endif
