// Stand-in: host-only compilation, no device qualifiers.
#pragma once
#define ONIKA_HOST_DEVICE_FUNC
#define ONIKA_DEVICE_FUNC
#define ONIKA_HOST_FUNC
#define ONIKA_CU_ATOMIC_ADD(x, a) ((x) += (a))
