// facade_test.cpp - the rsbd8.hpp facade used the way the reference's portable unit test uses
// the reference API (multiplatform/main.cpp), on device-resident arrays.  Known answers are
// checked here; with an output directory argument the random cases are written as raw
// files (inputs and outputs) for the Python test to compare with the oracle.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "rsbd8.hpp"

static int failures = 0;
#define CHECK(c)                                                                   \
    do {                                                                           \
        if (!(c)) {                                                                \
            std::fprintf(stderr, "CHECK failed at line %d: %s\n", __LINE__, #c);   \
            ++failures;                                                            \
        }                                                                          \
    } while (0)

template <typename T>
static T *todev(const std::vector<T> &h) {
    T *d = nullptr;
    cudaMalloc(reinterpret_cast<void **>(&d), h.size() * sizeof(T) + 1);
    cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}
template <typename T>
static std::vector<T> tohost(const T *d, std::size_t n) {
    std::vector<T> h(n);
    cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
    return h;
}

enum cert_v_binencoding64 : std::uint8_t { e0 = 0, ei = 18, eq = 26, eB = 37, eE = 40, eU = 56, e_ = 63 };

#pragma pack(push, 1)
class Testmeclass {
    std::uint64_t wasted{};
    char misalignoffset{};

public:
    std::uint64_t co;
    std::int64_t sco;
    std::uint64_t get() const noexcept { return co; }
    std::uint64_t getwparam(int testfor8in) const noexcept { return testfor8in == 8 ? co : 0; }
    std::int64_t sget() const noexcept { return sco; }
    Testmeclass(std::uint64_t input) noexcept : co{input}, sco{static_cast<std::int64_t>(input) - 1} {}
};
#pragma pack(pop)
static_assert(sizeof(Testmeclass) == 25, "packed test class");

struct Rec24 {
    std::uint64_t id;
    double key;
    std::uint32_t tag;
    std::uint32_t pad;
};

struct Rec4 {           // the records of oracle/ref_forms.cpp: id, then 32-bit keys a b c d
    std::uint64_t id;
    std::uint32_t a, b, c, d;
    // the getters of oracle/ref_forms.cpp: by value, by reference, by pointer, by pointer chosen by an argument
    std::uint32_t geta() const noexcept { return a; }
    std::uint32_t const &refa() const noexcept { return a; }
    std::uint32_t const *pointa() const noexcept { return &a; }
    std::uint32_t const *pick(int k) const noexcept { return k ? &c : &a; }
};

static std::uint64_t splitmix(std::uint64_t &s) {
    std::uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <typename T>
static void dump(const std::string &dir, const std::string &name, const std::vector<T> &v) {
    if (dir.empty()) return;
    FILE *f = std::fopen((dir + "/" + name).c_str(), "wb");
    std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

int main(int argc, char **argv) {
    const std::string outdir = argc > 1 ? argv[1] : "";
    {  // multiplatform/main.cpp:10-19: uint32, in place
        std::vector<std::uint32_t> h{18, 33, 21, 0, 5, 1, 13};
        std::uint32_t *d = todev(h);
        CHECK(rsbd8::radixsort(h.size(), d));
        CHECK((tohost(d, h.size()) == std::vector<std::uint32_t>{0, 1, 5, 13, 18, 21, 33}));
        cudaFree(d);
    }
    {  // multiplatform/main.cpp:191-198: single-byte enum, descending reverse and ascending
        std::vector<cert_v_binencoding64> tein{e0, eB, e_, ei, eq, eU, eE};
        auto *din = todev(tein);
        cert_v_binencoding64 *dout = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), 7);
        CHECK(rsbd8::radixsortcopy<rsbd8::sortingdirection::dscrevorder>(7, din, dout));
        CHECK((tohost(dout, 7) == std::vector<cert_v_binencoding64>{e_, eU, eE, eB, eq, ei, e0}));
        CHECK(rsbd8::radixsortcopy<rsbd8::sortingdirection::ascfwdorder>(7, din, dout));
        CHECK((tohost(dout, 7) == std::vector<cert_v_binencoding64>{e0, ei, eq, eB, eE, eU, e_}));
        cudaFree(din);
        cudaFree(dout);
    }
    std::uint32_t *doutm = nullptr;
    {  // multiplatform/main.cpp:201-205: float bit patterns, ascending
        std::vector<std::uint32_t> inm{8, 0, 3, 1u << 31 | 2, 3, 1u << 31 | 18, 1u << 31 | 2};
        auto *din = todev(inm);
        cudaMalloc(reinterpret_cast<void **>(&doutm), 7 * 4);
        CHECK(rsbd8::radixsortcopy(7, reinterpret_cast<float *>(din), reinterpret_cast<float *>(doutm)));
        CHECK((tohost(doutm, 7) ==
               std::vector<std::uint32_t>{1u << 31 | 18, 1u << 31 | 2, 1u << 31 | 2, 0, 3, 3, 8}));
        cudaFree(din);
    }
    {  // multiplatform/main.cpp:208-215: float pointers, descending reverse order, ties by address
        std::vector<float const *> inim{
            reinterpret_cast<float const *>(doutm + 6), reinterpret_cast<float const *>(doutm + 3),
            reinterpret_cast<float const *>(doutm + 4), reinterpret_cast<float const *>(doutm + 1),
            reinterpret_cast<float const *>(doutm + 5), reinterpret_cast<float const *>(doutm),
            reinterpret_cast<float const *>(doutm + 2)};
        auto *din = todev(inim);
        float const **dout = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), 7 * sizeof(void *));
        CHECK(rsbd8::radixsortcopy<rsbd8::sortingdirection::dscrevorder>(7, din, dout));
        auto o = tohost(dout, 7);
        CHECK(o[0] == inim[0] && o[1] == inim[4] && o[2] == inim[2] && o[3] == inim[1] && o[4] == inim[6] &&
              o[5] == inim[3] && o[6] == inim[5]);
        CHECK(rsbd8::radixsortcopy<rsbd8::sortingdirection::ascfwdorder>(7, din, dout));
        auto o2 = tohost(dout, 7);
        std::vector<std::uint32_t> vals(7);
        for (int i = 0; i < 7; ++i) cudaMemcpy(&vals[i], o2[i], 4, cudaMemcpyDeviceToHost);
        CHECK((vals == std::vector<std::uint32_t>{1u << 31 | 18, 1u << 31 | 2, 1u << 31 | 2, 0, 3, 3, 8}));
        cudaFree(din);
        cudaFree(dout);
    }
    cudaFree(doutm);
    {  // multiplatform/main.cpp:219-304: packed 25-byte class; getter, member and type+offset forms
        Testmeclass *objs = nullptr;   // managed: the host evaluates getters, the device reads members
        cudaMallocManaged(reinterpret_cast<void **>(&objs), 7 * sizeof(Testmeclass));
        const std::uint64_t vals[7]{8, 0, 6, 4, 0, 2, 6};
        for (int i = 0; i < 7; ++i) new (objs + i) Testmeclass(vals[i]);
        std::vector<Testmeclass const *> fin;
        for (int i = 0; i < 7; ++i) fin.push_back(objs + i);
        auto *din = todev(fin);
        Testmeclass const **dout = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), 7 * sizeof(void *));
        const std::vector<int> want{1, 4, 5, 3, 2, 6, 0};
        auto order = [&] {
            auto o = tohost(dout, 7);
            std::vector<int> idx;
            for (auto p : o) idx.push_back(int(p - objs));
            return idx;
        };
        CHECK((rsbd8::radixsortcopy<&Testmeclass::get>(7, din, dout)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<&Testmeclass::getwparam>(7, din, dout, 0, 8)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<&Testmeclass::co>(7, din, dout)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<std::uint64_t, 9>(7, din, dout)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<&Testmeclass::sget>(7, din, dout)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<&Testmeclass::sco>(7, din, dout)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<std::int64_t, 17>(7, din, dout)));
        CHECK(order() == want);
        CHECK((rsbd8::radixsortcopy<std::int64_t, 17, rsbd8::sortingdirection::dscrevorder>(7, din, dout)));
        CHECK((order() == std::vector<int>{0, 6, 2, 3, 5, 4, 1}));
        cudaFree(din);
        cudaFree(dout);
        cudaFree(objs);
    }
    {  // random cases for the oracle comparison: noalloc forms, modes, records by member
        const std::size_t n = 100003;
        std::uint64_t s = 12345;
        std::vector<float> f(n);
        for (auto &x : f) {
            std::uint32_t b = std::uint32_t(splitmix(s));
            if ((b & 63) == 0) b &= 0x80000000u;                 // +-0.0
            std::memcpy(&x, &b, 4);
        }
        auto *din = todev(f);
        float *dout = nullptr, *dbuf = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), n * 4);
        cudaMalloc(reinterpret_cast<void **>(&dbuf), n * 4);
        constexpr auto dsc = rsbd8::sortingdirection::dscrevorder;
        constexpr auto abs = rsbd8::sortingmode::nativeabs;
        void *scratch = nullptr;
        cudaMalloc(&scratch, rsbd8::gpuscratchbytes<dsc, abs, float>(n));
        rsbd8::radixsortcopynoalloc<dsc, abs>(n, 0u, nullptr, scratch, din, dout, dbuf);
        CHECK(rsbd8g_scratch_status(scratch, nullptr) == RSBD8G_OK);
        dump(outdir, "f32_in.bin", f);
        dump(outdir, "f32_nativeabs_dscrevorder.bin", tohost(dout, n));
        rsbd8::radixsortnoalloc<rsbd8::sortingdirection::ascrevorder>(n, scratch, din, dbuf, true);
        cudaDeviceSynchronize();
        dump(outdir, "f32_native_ascrevorder_movetobuffer.bin", tohost(dbuf, n));
        cudaFree(din);
        cudaFree(dout);
        cudaFree(dbuf);
        cudaFree(scratch);

        std::vector<Rec24> recs(n);
        for (std::size_t i = 0; i < n; ++i) {
            recs[i].id = i;
            std::uint64_t b = splitmix(s);
            recs[i].key = double(std::int64_t(b >> 11) - (std::int64_t(1) << 52)) / 1024.0;
            if (i > 0 && (b & 7) == 0) recs[i].key = recs[b % i].key;
        }
        auto *drec = todev(recs);
        std::vector<Rec24 *> ptrs(n);
        for (std::size_t i = 0; i < n; ++i) ptrs[i] = drec + i;
        auto *dp = todev(ptrs);
        Rec24 **dpo = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dpo), n * sizeof(void *));
        CHECK((rsbd8::radixsortcopy<&Rec24::key, rsbd8::sortingdirection::dscfwdorder>(n, dp, dpo)));
        auto po = tohost(dpo, n);
        std::vector<std::uint64_t> idx(n);
        for (std::size_t i = 0; i < n; ++i) idx[i] = std::uint64_t(po[i] - drec);
        std::vector<double> keys(n);
        for (std::size_t i = 0; i < n; ++i) keys[i] = recs[i].key;
        dump(outdir, "rec_keys.bin", keys);
        dump(outdir, "rec_member_dscfwdorder_idx.bin", idx);
        CHECK((rsbd8::radixsort<double, 8, rsbd8::sortingdirection::dscfwdorder>(n, dp)));
        auto pi = tohost(dp, n);
        for (std::size_t i = 0; i < n; ++i) if (std::uint64_t(pi[i] - drec) != idx[i]) { ++failures; break; }
        cudaFree(drec);
        cudaFree(dp);
        cudaFree(dpo);
    }
    {  // indexed / offset indirection forms (oracle/ref_forms.cpp runs the same calls on the reference);
       // each order is written as "<form>: i0 ... i5" for the comparison with tests/golden/ref_forms.json
        constexpr int n = 6;
        const std::uint32_t av[n]{5, 3, 9, 1, 7, 2}, bv[n]{10, 60, 20, 50, 30, 40}, cv[n]{6, 5, 4, 3, 2, 1},
            dv[n]{1, 3, 5, 2, 4, 6};
        std::vector<Rec4> h(n);
        for (int i = 0; i < n; ++i) h[i] = Rec4{std::uint64_t(i), av[i], bv[i], cv[i], dv[i]};
        Rec4 *drec = todev(h);
        std::vector<Rec4 *> hp(n);
        std::vector<std::uint32_t *> hk(n);
        for (int i = 0; i < n; ++i) {
            hp[i] = drec + i;
            hk[i] = &drec[i].a;
        }
        Rec4 **din = todev(hp), **dout = nullptr, **dbuf = nullptr;
        std::uint32_t **kin = todev(hk), **kout = nullptr, **kbuf = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), n * sizeof(void *));
        cudaMalloc(reinterpret_cast<void **>(&dbuf), n * sizeof(void *));
        cudaMalloc(reinterpret_cast<void **>(&kout), n * sizeof(void *));
        cudaMalloc(reinterpret_cast<void **>(&kbuf), n * sizeof(void *));
        void *scratch = nullptr;
        cudaMalloc(&scratch, rsbd8::gpuscratchbytesindirect<rsbd8::sortingdirection::ascfwdorder,
                                                            rsbd8::sortingmode::native, std::uint32_t>(n));
        std::string forms;
        auto show = [&](const char *t, Rec4 **d) {
            auto o = tohost(d, n);
            forms += t;
            forms += ":";
            for (auto p : o) forms += " " + std::to_string(p - drec);
            forms += "\n";
        };
        auto showk = [&](const char *t, std::uint32_t **d) {
            auto o = tohost(d, n);
            forms += t;
            forms += ":";
            for (auto p : o) forms += " " + std::to_string((reinterpret_cast<char *>(p) - 8 - reinterpret_cast<char *>(drec)) / 24);
            forms += "\n";
        };
        constexpr auto A = rsbd8::sortingdirection::ascfwdorder;
        constexpr auto D = rsbd8::sortingdirection::dscfwdorder;
        constexpr auto N = rsbd8::sortingmode::native;
        CHECK(rsbd8::radixsortcopy<&Rec4::a>(n, din, dout)); show("member a", dout);
        CHECK((rsbd8::radixsortcopy<&Rec4::a, A, N, 4>(n, din, dout))); show("member a, indirection2 4", dout);
        CHECK(rsbd8::radixsortcopy<&Rec4::a>(n, din, dout, 0, 1)); show("member a, index 1", dout);
        CHECK((rsbd8::radixsortcopy<&Rec4::a, A, N, 4>(n, din, dout, 0, 1))); show("member a, indirection2 4, index 1", dout);
        CHECK((rsbd8::radixsortcopy<&Rec4::a, A, N, 0, true>(n, din, dout, 0, 2))); show("member a, isindexed2, index 2", dout);
        CHECK((rsbd8::radixsortcopy<&Rec4::a, A, N, 4, true>(n, din, dout, 0, 1))); show("member a, indirection2 4, isindexed2, index 1", dout);
        // the noalloc form of the same call
        rsbd8::radixsortcopynoalloc<&Rec4::a, A, N, 0, true>(n, 0u, nullptr, scratch, din, dout, dbuf, 1, 2);
        show("member a, isindexed2, indices 1 2", dout);
        CHECK(rsbd8g_scratch_status(scratch, nullptr) == RSBD8G_OK);
        CHECK((rsbd8::radixsortcopy<&Rec4::a, D, N, 0, true>(n, din, dout, 0, 1, 2))); show("member a desc, isindexed2, indices 1 2", dout);
        CHECK((rsbd8::radixsortcopy<std::uint32_t, 8>(n, din, dout))); show("offset 8", dout);
        CHECK((rsbd8::radixsortcopy<std::uint32_t, 8, A, N, 4>(n, din, dout))); show("offset 8, indirection2 4", dout);
        CHECK((rsbd8::radixsortcopy<std::uint32_t, 8>(n, din, dout, 0, 2))); show("offset 8, index 2", dout);
        {   // in-place noalloc form, on a copy of the pointer array
            Rec4 **dwork = todev(hp);
            rsbd8::radixsortnoalloc<std::uint32_t, 8, A, N, 0, true>(n, 0u, nullptr, scratch, dwork, dbuf, false, 3);
            show("offset 8, isindexed2, index 3", dwork);
            cudaFree(dwork);
        }
        CHECK((rsbd8::radixsortcopy<A, N, 4>(n, kin, kout))); showk("second level, indirection2 4", kout);
        rsbd8::radixsortcopynoalloc<A, N, 0, true>(n, 0u, nullptr, scratch, kin, kout, kbuf, 2);
        showk("second level, isindexed2, index 2", kout);
        CHECK((rsbd8::radixsortcopy<A, N, 4, true>(n, kin, kout, 0, 1))); showk("second level, indirection2 4, isindexed2, index 1", kout);
        CHECK(rsbd8g_scratch_status(scratch, nullptr) == RSBD8G_OK);
        {   // getters: the host evaluates them on managed copies of the records
            Rec4 *mrec = nullptr;
            cudaMallocManaged(reinterpret_cast<void **>(&mrec), n * sizeof(Rec4));
            for (int i = 0; i < n; ++i) mrec[i] = h[i];
            std::vector<Rec4 *> mp(n);
            for (int i = 0; i < n; ++i) mp[i] = mrec + i;
            Rec4 **min = todev(mp);
            auto showm = [&](const char *t, Rec4 **d) {
                auto o = tohost(d, n);
                forms += t;
                forms += ":";
                for (auto p : o) forms += " " + std::to_string(p - mrec);
                forms += "\n";
            };
            CHECK(rsbd8::radixsortcopy<&Rec4::geta>(n, min, dout)); showm("getter a", dout);
            CHECK((rsbd8::radixsortcopy<&Rec4::geta, D>(n, min, dout))); showm("getter a desc", dout);
            CHECK((rsbd8::radixsortcopy<&Rec4::refa, A, N, 4>(n, min, dout))); showm("getter reference a, indirection2 4", dout);
            CHECK((rsbd8::radixsortcopy<&Rec4::pointa, A, N, 0, true>(n, min, dout, 0, 2)));
            showm("getter pointer a, isindexed2, index 2", dout);
            // the noalloc forms of getters: the keys go to the tail of the scratch
            void *gscratch = nullptr;
            cudaMalloc(&gscratch, rsbd8::gpuscratchbytesgetter<D, N, std::uint32_t>(n));
            rsbd8::radixsortcopynoalloc<&Rec4::pointa, D, N, 4, true>(n, 0u, nullptr, gscratch, min, dout, dbuf, 2);
            CHECK(rsbd8g_scratch_status(gscratch, nullptr) == RSBD8G_OK);
            showm("getter pointer a desc, indirection2 4, isindexed2, index 2", dout);
            {
                Rec4 **mwork = todev(mp);
                rsbd8::radixsortnoalloc<&Rec4::pick, A, N, 0, true>(n, 0u, nullptr, gscratch, mwork, dbuf, false, 1, 1);
                CHECK(rsbd8g_scratch_status(gscratch, nullptr) == RSBD8G_OK);
                showm("getter pick(1), isindexed2, index 1", mwork);
                cudaFree(mwork);
            }
            CHECK((rsbd8::radixsortcopy<&Rec4::pick, A, N, 4>(n, min, dout, 0, 0))); showm("getter pick(0), indirection2 4", dout);
            cudaFree(gscratch);
            cudaFree(min);
            cudaFree(mrec);
        }
        std::fputs(forms.c_str(), stdout);
        if (!outdir.empty()) {
            FILE *f = std::fopen((outdir + "/forms.txt").c_str(), "w");
            std::fputs(forms.c_str(), f);
            std::fclose(f);
        }
        cudaFree(drec);
        cudaFree(din);
        cudaFree(dout);
        cudaFree(dbuf);
        cudaFree(kin);
        cudaFree(kout);
        cudaFree(kbuf);
        cudaFree(scratch);
    }
    {  // 8-bit keys: the single-part noalloc forms (no buffer argument)
        std::vector<std::int8_t> h{5, -3, 9, -128, 127, 0, -3, 5};
        std::int8_t *din = todev(h), *dout = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), h.size());
        void *scratch = nullptr;
        cudaMalloc(&scratch, rsbd8::gpuscratchbytes<rsbd8::sortingdirection::ascfwdorder, rsbd8::sortingmode::native,
                                                    std::int8_t>(h.size()));
        rsbd8::radixsortcopynoalloc(h.size(), 0u, nullptr, scratch, din, dout);
        CHECK((tohost(dout, h.size()) == std::vector<std::int8_t>{-128, -3, -3, 0, 5, 5, 9, 127}));
        rsbd8::radixsortnoalloc<rsbd8::sortingdirection::dscfwdorder>(h.size(), 0u, nullptr, scratch, din);
        CHECK((tohost(din, h.size()) == std::vector<std::int8_t>{127, 9, 5, 5, 0, -3, -3, -128}));
        CHECK(rsbd8g_scratch_status(scratch, nullptr) == RSBD8G_OK);
        cudaFree(din);
        cudaFree(dout);
        cudaFree(scratch);
    }
    {  // 16-byte keys: long double (x87 in 16 bytes on x86-64, binary128 on AArch64) and 128-bit integers
        const std::size_t n = 5003;
        std::uint64_t s = 777;
        std::vector<long double> h(n);
        for (std::size_t i = 0; i < n; ++i) {
            const std::int64_t v = std::int64_t(splitmix(s) % 2001) - 1000;     // many ties
            h[i] = (i % 11 == 0) ? (i % 22 == 0 ? -0.0L : 0.0L) : static_cast<long double>(v) / 7.0L;
        }
        long double *din = todev(h), *dout = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dout), n * sizeof(long double));
        CHECK(rsbd8::radixsortcopy(n, din, dout));
        std::vector<long double> want = h;
        std::stable_sort(want.begin(), want.end(), [](long double a, long double b) { return a < b; });
        const auto got = tohost(dout, n);
        bool same = true;
        for (std::size_t i = 0; i < n; ++i)
            same &= got[i] == want[i] && std::signbit(got[i]) == std::signbit(want[i]);   // -0 and +0 tie, stably
        CHECK(same);
        CHECK(rsbd8::radixsortcopy<rsbd8::sortingdirection::dscfwdorder>(n, din, dout));
        std::stable_sort(want.begin(), want.end(), [](long double a, long double b) { return b < a; });
        std::stable_sort(h.begin(), h.end(), [](long double a, long double b) { return b < a; });
        const auto got2 = tohost(dout, n);
        same = true;
        for (std::size_t i = 0; i < n; ++i) same &= got2[i] == h[i] && std::signbit(got2[i]) == std::signbit(h[i]);
        CHECK(same);
        cudaFree(din);
        cudaFree(dout);
#ifdef __SIZEOF_INT128__
        std::vector<__int128> q(n);
        for (auto &x : q) x = (__int128(std::int64_t(splitmix(s))) << 64) | __int128(splitmix(s) % 5);
        __int128 *dq = todev(q), *dqo = nullptr;
        cudaMalloc(reinterpret_cast<void **>(&dqo), n * 16);
        CHECK(rsbd8::radixsortcopy<rsbd8::sortingdirection::dscfwdorder>(n, dq, dqo));
        std::vector<__int128> qw = q;
        std::stable_sort(qw.begin(), qw.end(), [](__int128 a, __int128 b) { return b < a; });
        CHECK(tohost(dqo, n) == qw);
        CHECK(rsbd8::radixsort(n, reinterpret_cast<unsigned __int128 *>(dq)));
        std::vector<unsigned __int128> qu(q.begin(), q.end());
        std::stable_sort(qu.begin(), qu.end());
        CHECK(tohost(reinterpret_cast<unsigned __int128 *>(dq), n) == qu);
        cudaFree(dq);
        cudaFree(dqo);
#endif
    }
    std::printf("%s (%d failures)\n", failures ? "FAIL" : "PASS", failures);
    return failures ? 1 : 0;
}
