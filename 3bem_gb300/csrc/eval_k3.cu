#define EVAL_KID 3
#include "eval_inst.cuh"
