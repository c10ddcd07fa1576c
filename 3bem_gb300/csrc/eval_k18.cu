#define EVAL_KID 18
#define EVAL_FP64_ONLY 1
#include "eval_inst.cuh"
