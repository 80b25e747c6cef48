/* include-name shim: the Peristalsis kernels include the utility in lower case */
#include "PeristalsisUtil.cu"
