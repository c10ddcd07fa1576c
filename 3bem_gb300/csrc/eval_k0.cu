#define EVAL_KID 0
#include "eval_inst.cuh"
