#define EVAL_KID 4
#include "eval_inst.cuh"
