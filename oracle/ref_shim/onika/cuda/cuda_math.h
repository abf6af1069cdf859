#pragma once
#include <cmath>
#include <onika/cuda/cuda.h>
