// IF4: evolve and coefficient launchers.
#define RK_METHOD_ID RK_IF4
#define RK_METHOD_NAME IF4
#include "rk_launch_impl.cuh"
