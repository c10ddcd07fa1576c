#define EVAL_KID 23
#define EVAL_FP64_ONLY 1
#include "eval_inst.cuh"
