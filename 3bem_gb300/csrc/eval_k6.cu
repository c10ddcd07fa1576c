#define EVAL_KID 6
#include "eval_inst.cuh"
