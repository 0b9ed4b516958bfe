/* cuda_runtime_api.h stand-in for the oracle host build */
#include "cudashim.h"
