/* glibc no longer ships <sys/sysctl.h>; pbrt's parallel.cpp includes it but
 * uses it only on BSD/macOS. */
#ifndef ORACLE_REF_SHIM_SYSCTL_H
#define ORACLE_REF_SHIM_SYSCTL_H
#endif
