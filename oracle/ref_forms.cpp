// ref_forms.cpp - test infrastructure: runs the reference's own rsbd8::radixsortcopy on the
// indirection call forms whose key position depends on indirection2 and index arguments
// (Radixsortbidi8.hpp:2412-2470 splitgetobject, :2740-2770 indirectinput1, :2787-2813
// indirectinput2) and prints the resulting element order of each form, one line per form:
//     <form name>: i0 i1 ... i5
// tests/golden/make_ref_forms.py turns the output into tests/golden/ref_forms.json, the
// known answers the facade's GPU test checks.  Built by `make -C oracle ref` where the reference
// header exists; it only includes the header (nothing is copied from it).
#include "Radixsortbidi8.hpp"

#include <cstdint>
#include <cstdio>

struct Rec {            // 24 bytes: id, then four 32-bit keys a b c d at bytes 8, 12, 16, 20
    std::uint64_t id;
    std::uint32_t a, b, c, d;
    // getters: by value, by reference, by pointer, and by pointer chosen by an argument
    std::uint32_t geta() const noexcept { return a; }
    std::uint32_t const &refa() const noexcept { return a; }
    std::uint32_t const *pointa() const noexcept { return &a; }
    std::uint32_t const *pick(int k) const noexcept { return k ? &c : &a; }
};

int main() {
    constexpr int n = 6;
    static Rec s[n];
    const std::uint32_t av[n]{5, 3, 9, 1, 7, 2}, bv[n]{10, 60, 20, 50, 30, 40}, cv[n]{6, 5, 4, 3, 2, 1},
        dv[n]{1, 3, 5, 2, 4, 6};
    for (int i = 0; i < n; ++i) s[i] = Rec{std::uint64_t(i), av[i], bv[i], cv[i], dv[i]};
    Rec *in[n], *out[n];
    std::uint32_t *kin[n], *kout[n];
    for (int i = 0; i < n; ++i) {
        in[i] = s + i;
        kin[i] = &s[i].a;
    }
    auto show = [&](const char *t) {
        std::printf("%s:", t);
        for (int i = 0; i < n; ++i) std::printf(" %d", int(out[i]->id));
        std::printf("\n");
    };
    auto showk = [&](const char *t) {
        std::printf("%s:", t);
        for (int i = 0; i < n; ++i) std::printf(" %d", int(reinterpret_cast<Rec *>(reinterpret_cast<char *>(kout[i]) - 8)->id));
        std::printf("\n");
    };
    constexpr auto A = rsbd8::sortingdirection::ascfwdorder;
    constexpr auto D = rsbd8::sortingdirection::dscfwdorder;
    constexpr auto N = rsbd8::sortingmode::native;
    constexpr int F = MAP_ANONYMOUS | MAP_PRIVATE;
    bool ok = true;
    ok &= rsbd8::radixsortcopy<&Rec::a>(n, in, out); show("member a");
    ok &= rsbd8::radixsortcopy<&Rec::a, A, N, 4>(n, in, out); show("member a, indirection2 4");
    ok &= rsbd8::radixsortcopy<&Rec::a>(n, in, out, F, 1); show("member a, index 1");
    ok &= rsbd8::radixsortcopy<&Rec::a, A, N, 4>(n, in, out, F, 1); show("member a, indirection2 4, index 1");
    ok &= rsbd8::radixsortcopy<&Rec::a, A, N, 0, true>(n, in, out, F, 2); show("member a, isindexed2, index 2");
    ok &= rsbd8::radixsortcopy<&Rec::a, A, N, 4, true>(n, in, out, F, 1); show("member a, indirection2 4, isindexed2, index 1");
    ok &= rsbd8::radixsortcopy<&Rec::a, A, N, 0, true>(n, in, out, F, 1, 2); show("member a, isindexed2, indices 1 2");
    ok &= rsbd8::radixsortcopy<&Rec::a, D, N, 0, true>(n, in, out, F, 1, 2); show("member a desc, isindexed2, indices 1 2");
    ok &= rsbd8::radixsortcopy<std::uint32_t, 8>(n, in, out); show("offset 8");
    ok &= rsbd8::radixsortcopy<std::uint32_t, 8, A, N, 4>(n, in, out); show("offset 8, indirection2 4");
    ok &= rsbd8::radixsortcopy<std::uint32_t, 8>(n, in, out, F, 2); show("offset 8, index 2");
    ok &= rsbd8::radixsortcopy<std::uint32_t, 8, A, N, 0, true>(n, in, out, F, 3); show("offset 8, isindexed2, index 3");
    ok &= rsbd8::radixsortcopy<A, N, 4>(n, kin, kout); showk("second level, indirection2 4");
    ok &= rsbd8::radixsortcopy<A, N, 0, true>(n, kin, kout, F, 2); showk("second level, isindexed2, index 2");
    ok &= rsbd8::radixsortcopy<A, N, 4, true>(n, kin, kout, F, 1); showk("second level, indirection2 4, isindexed2, index 1");
    ok &= rsbd8::radixsortcopy<&Rec::geta>(n, in, out); show("getter a");
    ok &= rsbd8::radixsortcopy<&Rec::geta, D>(n, in, out); show("getter a desc");
    ok &= rsbd8::radixsortcopy<&Rec::refa, A, N, 4>(n, in, out); show("getter reference a, indirection2 4");
    ok &= rsbd8::radixsortcopy<&Rec::pointa, A, N, 0, true>(n, in, out, F, 2); show("getter pointer a, isindexed2, index 2");
    ok &= rsbd8::radixsortcopy<&Rec::pointa, D, N, 4, true>(n, in, out, F, 2); show("getter pointer a desc, indirection2 4, isindexed2, index 2");
    ok &= rsbd8::radixsortcopy<&Rec::pick, A, N, 0, true>(n, in, out, F, 1, 1); show("getter pick(1), isindexed2, index 1");
    ok &= rsbd8::radixsortcopy<&Rec::pick, A, N, 4>(n, in, out, F, 0); show("getter pick(0), indirection2 4");
    std::printf("all calls returned true: %d\n", ok ? 1 : 0);
    return ok ? 0 : 1;
}
