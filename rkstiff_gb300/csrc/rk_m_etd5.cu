// ETD5: evolve and coefficient launchers.
#define RK_METHOD_ID RK_ETD5
#define RK_METHOD_NAME ETD5
#include "rk_launch_impl.cuh"
