/* Stand-in for the xobjects atomic-add header (unused on the CPU oracle).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef XTG_REF_SHIM_ATOMICADD_H
#define XTG_REF_SHIM_ATOMICADD_H
#endif
