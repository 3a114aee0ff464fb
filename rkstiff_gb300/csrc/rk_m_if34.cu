// IF34: evolve and coefficient launchers.
#define RK_METHOD_ID RK_IF34
#define RK_METHOD_NAME IF34
#include "rk_launch_impl.cuh"
