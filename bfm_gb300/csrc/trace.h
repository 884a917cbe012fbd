/* NVTX ranges around the library's entry points and their phases, so that a
 * timeline (Nsight Systems) or a kernel profile filtered by range (Nsight
 * Compute --nvtx) shows which call and which phase a kernel belongs to.
 * NVTX v3 is header-only: with no tool attached, a push or pop costs a test
 * of one function pointer. */
#pragma once

#include <nvtx3/nvToolsExt.h>

#define BFM_RANGE_PUSH(name) nvtxRangePushA(name)
#define BFM_RANGE_POP() nvtxRangePop()

#ifdef __cplusplus
/* a range that ends where the enclosing scope ends (every return path) */
struct BfmRange {
	explicit BfmRange(const char* name) { nvtxRangePushA(name); }
	~BfmRange() { nvtxRangePop(); }
	BfmRange(const BfmRange&) = delete;
	BfmRange& operator=(const BfmRange&) = delete;
};
#define BFM_RANGE_CAT2(a, b) a##b
#define BFM_RANGE_CAT(a, b) BFM_RANGE_CAT2(a, b)
#define BFM_RANGE(name) BfmRange const BFM_RANGE_CAT(bfm_range_, __LINE__)(name)
#endif
