/* Stand-in for the system-types header that the reference's type headers
 * include as ../dunelib/lib_sys_types.h (a path the reference does not have).
 * Same typedefs as the reference's lib/lib_sys_types.h; C11 allows the repeat. */
#pragma once
#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <sys/types.h>
typedef unsigned int uint;
typedef unsigned short ushort;
typedef unsigned long ulong;
typedef unsigned char uchar;
