// prelude.cuh -- system headers the reference's parameter files include,
// included first so that the header settings below (`#define float double`
// around the parameter file: the sweep scripts' `typedef double
// highprecision`) touch only the reference's own declarations.
#pragma once
#include <stdio.h>
#include <stdlib.h>
#include <iostream>
#include <cuda.h>
#include <cuda_runtime.h>
#include <unistd.h>
#include <fstream>
#include <string>
#include <sstream>
#include <mma.h>
#include <device_launch_parameters.h>
#include <cuda_fp16.h>
#include <math.h>
#include <algorithm>
