#define EVAL_KID 2
#include "eval_inst.cuh"
