// fyg_batch.cu -- uneven-length batches (many transforms of different lengths, packed back to
// back).  No counterpart in the reference, which runs one transform per dispatch call.
#include <algorithm>
#include <map>
#include <memory>
#include <vector>

#include "fyg_host.h"

struct fyg_batch {
    std::vector<size_t> lengths;
    std::vector<int64_t> offsets;     // packed offsets (elements)
    int dtype = FYG_C32;
    int flags = 0;
    std::map<size_t, fyg_plan*> plans; // one batch-1 plan per distinct length
    ~fyg_batch() {
        for (auto& kv : plans) fyg_plan_destroy(kv.second);
    }
};

using namespace fyg;

extern "C" {

int fyg_batch_create(const size_t* lengths, size_t count, int dtype, int flags, fyg_batch** out) {
    clear_error();
    if (!out || (!lengths && count)) return set_error(FYG_ERR_NULL_PTR, "null argument");
    *out = nullptr;
    if (dtype != FYG_C32 && dtype != FYG_C64) return set_error(FYG_ERR_INVALID_ARG, "bad dtype");
    auto b = std::make_unique<fyg_batch>();
    b->dtype = dtype;
    b->flags = flags;
    int64_t off = 0;
    for (size_t i = 0; i < count; ++i) {
        if (lengths[i] < 1) return set_error(FYG_ERR_INVALID_LENGTH, "length must be >= 1");
        b->lengths.push_back(lengths[i]);
        b->offsets.push_back(off);
        off += (int64_t)lengths[i];
        if (!b->plans.count(lengths[i])) {
            fyg_plan* p = nullptr;
            int rc = fyg_plan_create(lengths[i], dtype, 1, flags, &p);
            if (rc) return rc;
            b->plans[lengths[i]] = p;
        }
    }
    *out = b.release();
    return FYG_OK;
}

int fyg_batch_destroy(fyg_batch* batch) {
    delete batch;
    return FYG_OK;
}

int fyg_batch_execute_plain(fyg_batch* b, const void* in, void* out, int direction, void* stream) {
    clear_error();
    if (!b || !in || !out) return set_error(FYG_ERR_NULL_PTR, "null argument");
    const size_t eb = b->dtype == FYG_C32 ? 8 : 16;
    for (size_t i = 0; i < b->lengths.size(); ++i) {
        const char* x = (const char*)in + b->offsets[i] * eb;
        char* y = (char*)out + b->offsets[i] * eb;
        int rc = fyg_execute(b->plans[b->lengths[i]], x, y, direction, stream);
        if (rc) return rc;
    }
    return FYG_OK;
}

int fyg_batch_execute(fyg_batch* b, const void* in, void* out, const int64_t* offsets_dev, int direction,
                      void* stream) {
    (void)offsets_dev;
    return fyg_batch_execute_plain(b, in, out, direction, stream);
}

}  // extern "C"
