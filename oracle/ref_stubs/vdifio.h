/* Stand-in for vdifio's header type (a VDIF frame header is eight 32-bit
 * words, 32 bytes). Oracle harness use only. */
#ifndef VGB_STUB_VDIFIO_H
#define VGB_STUB_VDIFIO_H
#include <stdint.h>
#define VDIF_HEADER_BYTES 32
typedef struct vdif_header { uint32_t words[8]; } vdif_header;
#endif
