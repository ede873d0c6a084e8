// Second-order kernels for 1 general direction(s) at once (epg_second.cuh);
// one translation unit per table so they compile in parallel.
#include "epg_second.cuh"

namespace tsg {

extern const SecondEntry kSecondK1[];
extern const int kSecondK1Count;

const SecondEntry kSecondK1[] = {
    TSG_SECOND_ENTRY(4, 1, 1, 0),
    TSG_SECOND_ENTRY(4, 2, 1, 0),
    TSG_SECOND_ENTRY(4, 3, 1, 0),
    TSG_SECOND_ENTRY(4, 4, 1, 0),
    TSG_SECOND_ENTRY(4, 5, 1, 0),
    TSG_SECOND_ENTRY(4, 8, 1, 0),
    TSG_SECOND_ENTRY(4, 16, 1, 0),
    TSG_SECOND_ENTRY(2, 2, 1, 0),
    TSG_SECOND_ENTRY(2, 4, 1, 0),
    TSG_SECOND_ENTRY(2, 5, 1, 0),
    TSG_SECOND_ENTRY(2, 8, 1, 0),
    TSG_SECOND_ENTRY(2, 10, 1, 0),
    TSG_SECOND_ENTRY(2, 16, 1, 0),
    TSG_SECOND_ENTRY(2, 32, 1, 0),
};
const int kSecondK1Count = int(sizeof(kSecondK1) / sizeof(kSecondK1[0]));

}  // namespace tsg
