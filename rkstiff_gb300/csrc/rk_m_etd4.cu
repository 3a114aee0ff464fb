// ETD4: evolve and coefficient launchers.
#define RK_METHOD_ID RK_ETD4
#define RK_METHOD_NAME ETD4
#include "rk_launch_impl.cuh"
