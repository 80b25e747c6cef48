/* include-name shim: PeristalsisKernel.cu includes the header in lower case */
#include "PeristalsisKernel.cuh"
