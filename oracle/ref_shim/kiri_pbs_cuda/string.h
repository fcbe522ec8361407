/* Host-build shim for the reference harness: the reference's helper_string.h
 * includes <kiri_pbs_cuda/string.h>; the intended header is the C library's. */
#include <string.h>
