// Stand-in for the two OptiX names that the reference's utils/exception.h
// uses.  The CPU early-break path never calls OptiX.
#pragma once
typedef int OptixResult;
#define OPTIX_SUCCESS 0
inline const char* optixGetErrorName(OptixResult) { return "OPTIX_SHIM"; }
