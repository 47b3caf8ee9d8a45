/*
 * Stand-in for the xobjects runtime header that the reference's element
 * code includes (xtrack/headers/track.h:9). xobjects is not part of the
 * reference tree; this file defines the handful of macros the in-scope
 * element headers use so that they compile with a plain C compiler for the
 * reference-compiled CPU oracle. TEST INFRASTRUCTURE ONLY.
 */
#ifndef XTG_REF_SHIM_COMMON_H
#define XTG_REF_SHIM_COMMON_H

#include <math.h>
#include <stdint.h>
#include <stddef.h>

#define GPUFUN static inline
#define GPUKERN
#define GPUGLMEM
#define GPUSHAREDMEM
#define RESTRICT

#define POW2(X) ((X)*(X))
#define POW3(X) ((X)*(X)*(X))
#define POW4(X) ((X)*(X)*(X)*(X))
#define NONZERO(X) ((X) != 0.0)

#endif
