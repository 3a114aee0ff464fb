// ETD34: evolve and coefficient launchers.
#define RK_METHOD_ID RK_ETD34
#define RK_METHOD_NAME ETD34
#include "rk_launch_impl.cuh"
