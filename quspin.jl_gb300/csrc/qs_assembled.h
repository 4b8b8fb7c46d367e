// qs_assembled.h -- device storage of an assembled operator (see qs_assembled.cu).
#pragma once

#include <cstdint>

namespace qs {

struct Assembled {
    DevBuf rowptr;     // int64, n + 1
    DevBuf words;      // uint32 (column << code_bits) | code, when packed
    DevBuf cols;       // int32 column per nonzero, when not packed
    DevBuf codes;      // uint16 code per nonzero, when not packed
    DevBuf table64;    // complex double value per code
    DevBuf table32;    // complex float value per code
    DevBuf table_df;   // per code: re hi, re lo, im hi, im lo (float)
    DevBuf xsplit;     // x split into float pairs for the double-float product
    int64_t nnz = 0;
    int ncodes = 0;
    int code_bits = 0;
    bool packed = true;
    int lanes = 8;     // threads per row in the SpMV
};

}  // namespace qs
