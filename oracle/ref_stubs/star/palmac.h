/* Stand-in for PAL's macro header (the reference only uses it when
 * PAL_FOUND is defined, which the oracle harness does not define). */
#ifndef VGB_STUB_PALMAC_H
#define VGB_STUB_PALMAC_H
#endif
