#define EVAL_KID 1
#include "eval_inst.cuh"
