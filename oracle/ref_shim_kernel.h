/* Force-included when the reference's OpenCL C kernel
 * (FPGA/code/device/align_swi.cl) is compiled as host C by build_ref.sh:
 * maps the OpenCL C dialect onto C.  TEST INFRASTRUCTURE ONLY. */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
typedef unsigned char uchar;
typedef unsigned int uint;
typedef unsigned long ulong;
/* the device header's `typedef char int8_t` clashes with <stdint.h> */
#define int8_t ref_device_int8_t
#define __kernel
#define __global
