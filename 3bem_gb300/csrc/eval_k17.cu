#define EVAL_KID 17
#define EVAL_FP64_ONLY 1
#include "eval_inst.cuh"
