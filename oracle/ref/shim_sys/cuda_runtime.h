/* cuda_runtime.h stand-in for the oracle host build */
#include "cudashim.h"
