/* Stand-in for mwa_hyperbeam's opaque beam handle. Oracle harness use only. */
#ifndef VGB_STUB_HYPERBEAM_H
#define VGB_STUB_HYPERBEAM_H
typedef struct FEEBeam FEEBeam;
#endif
