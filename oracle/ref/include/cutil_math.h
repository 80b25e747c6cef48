/* include-name shim: the Peristalsis sources include "cutil_math.h" (CUDA SDK <= 4) */
#include "helper_math.h"
