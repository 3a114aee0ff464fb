// IF45DP: evolve and coefficient launchers.
#define RK_METHOD_ID RK_IF45DP
#define RK_METHOD_NAME IF45DP
#include "rk_launch_impl.cuh"
