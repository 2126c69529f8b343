/* device_launch_parameters.h — see cuda_runtime.h in this directory. */
#include "cuda_runtime.h"
