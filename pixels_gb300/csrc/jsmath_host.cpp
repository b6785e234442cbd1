// Host build of jsmath.cuh, exported for tests that compare the device math
// routines (same source, same operation sequence) with mpmath and libm.
#include "jsmath.cuh"
extern "C" {
double px_host_sin(double x) { return px_sin(x); }
double px_host_atan2(double y, double x) { return px_atan2(y, x); }
double px_host_hypot2(double a, double b) { return px_hypot2(a, b); }
double px_host_round(double x) { return px_round(x); }
}
