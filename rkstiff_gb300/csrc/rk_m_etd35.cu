// ETD35: evolve and coefficient launchers.
#define RK_METHOD_ID RK_ETD35
#define RK_METHOD_NAME ETD35
#include "rk_launch_impl.cuh"
