// Compile-time dispatch over the (multipole order, field order) pairs that the
// near-field and direct-sum kernels are instantiated for (0..2 each).
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
