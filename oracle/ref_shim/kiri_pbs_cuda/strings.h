/* Host-build shim for the reference harness (see string.h beside this file). */
#include <strings.h>
