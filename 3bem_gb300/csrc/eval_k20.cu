#define EVAL_KID 20
#define EVAL_FP64_ONLY 1
#include "eval_inst.cuh"
