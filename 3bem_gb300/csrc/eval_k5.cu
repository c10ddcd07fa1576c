#define EVAL_KID 5
#include "eval_inst.cuh"
