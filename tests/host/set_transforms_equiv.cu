// cgb_layers_set_transforms: one call over a long id list (checked and applied
// by the host thread pool when it can be) leaves the same host state as the
// same items applied in calls of 5,000 (the sequential loop), including the
// lists that must take the sequential loop: an absent layer, ids out of order,
// an identity transform, a scale error in the middle.  Host only: the handle's
// host state is built directly, without a device.
#include "host_state.cuh"
#include <random>
extern "C" cgb_status cgb_layers_set_transforms(cgb_composition*, size_t, const uint32_t*, const float*, uint32_t);
static cgb_composition* make(size_t N) {
    auto* c = new cgb_composition();
    c->layers.resize(N);
    c->layer_recs.resize(N);
    for (size_t i = 0; i < N; i++) {
        c->layers[i].present = (i % 97) != 5;
        c->layers[i].has_transform = (i % 89) != 7;
        c->layers[i].unchanged = 0xFFu;
        float t[6] = {0.9f, 0.1f, -0.1f, 0.9f, (float)i, 4.f};
        std::memcpy(c->layers[i].t, t, sizeof(t));
        std::memcpy(c->layer_recs[i].t, t, sizeof(t));
    }
    return c;
}
static bool same(cgb_composition* a, cgb_composition* b) {
    if (a->dirty_lo != b->dirty_lo || a->dirty_hi != b->dirty_hi || a->layers.size() != b->layers.size()) return false;
    for (size_t i = 0; i < a->layers.size(); i++) {
        if (std::memcmp(a->layers[i].t, b->layers[i].t, 24) || a->layers[i].unchanged != b->layers[i].unchanged ||
            a->layers[i].has_transform != b->layers[i].has_transform ||
            std::memcmp(a->layer_recs[i].t, b->layer_recs[i].t, 24) || a->layer_recs[i].flags != b->layer_recs[i].flags)
            return false;
    }
    return true;
}
int main() {
    const size_t N = 60000;
    std::mt19937 rng(7);
    int fails = 0;
    for (int sc = 0; sc < 6; sc++) {
        cgb_composition* a = make(N);
        cgb_composition* b = make(N);
        std::vector<uint32_t> ids;
        for (uint32_t i = 0; i < N; i++) if (sc == 0 || (i % 97) != 5) if (rng() % 10 < 9) ids.push_back(i);
        std::vector<float> tr(6 * ids.size());
        for (size_t k = 0; k < ids.size(); k++) {
            float t[6] = {0.9f, 0.1f, -0.1f, 0.9f, (float)ids[k] + ((rng() % 3) ? 0.5f : 0.f), 4.f};
            std::memcpy(&tr[6 * k], t, 24);
        }
        if (sc == 2) std::swap(ids[100], ids[101]);                 // not increasing
        if (sc == 3) { float t[6] = {1, 0, 0, 1, 0, 0}; std::memcpy(&tr[6 * 300], t, 24); }  // identity
        if (sc == 4) tr[6 * 40000] = 1.5f;                          // scale error in the middle
        // sc 0: includes absent layers; sc 1: plain; sc 5: plain, second call with the same values
        cgb_status sa = cgb_layers_set_transforms(a, ids.size(), ids.data(), tr.data(), 0);
        cgb_status sb = CGB_OK;
        for (size_t o = 0; o < ids.size() && sb == CGB_OK; o += 5000)
            sb = cgb_layers_set_transforms(b, std::min<size_t>(5000, ids.size() - o), ids.data() + o, tr.data() + 6 * o, 0);
        if (sc == 5) {
            sa = cgb_layers_set_transforms(a, ids.size(), ids.data(), tr.data(), 0);
            for (size_t o = 0; o < ids.size(); o += 5000)
                cgb_layers_set_transforms(b, std::min<size_t>(5000, ids.size() - o), ids.data() + o, tr.data() + 6 * o, 0);
        }
        const bool eq = sa == sb && same(a, b);
        printf("case %d: status %d/%d, %s\n", sc, (int)sa, (int)sb, eq ? "same" : "DIFFERENT");
        fails += !eq;
    }
    return fails;
}
