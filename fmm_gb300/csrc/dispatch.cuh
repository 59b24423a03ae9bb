// Compile-time dispatch over the (multipole order, field order) pairs that the
// near-field and direct-sum kernels are instantiated for: 0..2 each for the
// FP32 kernels (FMM_MF_SWITCH), 0..3 each for the FP64 ones
// (FMM_MF_SWITCH_F64).
#pragma once

#define FMM_MF_SWITCH(M_, F_, BODY)      \
    switch ((M_) * 3 + (F_)) {           \
        case 0: { constexpr int MM = 0, FF = 0; BODY; } break; \
        case 1: { constexpr int MM = 0, FF = 1; BODY; } break; \
        case 2: { constexpr int MM = 0, FF = 2; BODY; } break; \
        case 3: { constexpr int MM = 1, FF = 0; BODY; } break; \
        case 4: { constexpr int MM = 1, FF = 1; BODY; } break; \
        case 5: { constexpr int MM = 1, FF = 2; BODY; } break; \
        case 6: { constexpr int MM = 2, FF = 0; BODY; } break; \
        case 7: { constexpr int MM = 2, FF = 1; BODY; } break; \
        case 8: { constexpr int MM = 2, FF = 2; BODY; } break; \
        default: return FMM_ENOTSUP;     \
    }                                    \
    count_launches(1);

#define FMM_MF_SWITCH_F64(M_, F_, BODY)  \
    if ((M_) < 0 || (M_) > 3 || (F_) < 0 || (F_) > 3) return FMM_ENOTSUP; \
    switch ((M_) * 4 + (F_)) {           \
        case 0: { constexpr int MM = 0, FF = 0; BODY; } break; \
        case 1: { constexpr int MM = 0, FF = 1; BODY; } break; \
        case 2: { constexpr int MM = 0, FF = 2; BODY; } break; \
        case 3: { constexpr int MM = 0, FF = 3; BODY; } break; \
        case 4: { constexpr int MM = 1, FF = 0; BODY; } break; \
        case 5: { constexpr int MM = 1, FF = 1; BODY; } break; \
        case 6: { constexpr int MM = 1, FF = 2; BODY; } break; \
        case 7: { constexpr int MM = 1, FF = 3; BODY; } break; \
        case 8: { constexpr int MM = 2, FF = 0; BODY; } break; \
        case 9: { constexpr int MM = 2, FF = 1; BODY; } break; \
        case 10: { constexpr int MM = 2, FF = 2; BODY; } break; \
        case 11: { constexpr int MM = 2, FF = 3; BODY; } break; \
        case 12: { constexpr int MM = 3, FF = 0; BODY; } break; \
        case 13: { constexpr int MM = 3, FF = 1; BODY; } break; \
        case 14: { constexpr int MM = 3, FF = 2; BODY; } break; \
        default: { constexpr int MM = 3, FF = 3; BODY; } break; \
    }                                    \
    count_launches(1);
