// A caller written against the reference's C++ object API (sdbf_class.h /
// sdbf_set.h), compiled here against the GB300 compatibility headers and
// linked with libsdbf_gb300.so instead of the reference's libsdbf.a.
//
// usage: sdbf_api_demo <fileA> <fileB> <set.sdbf>
//   prints: stream digest of A, 16 KiB block digest of B, A-vs-B score,
//   the score after a to_string() / parse round trip, then the set's
//   compare_all_quiet(threshold 1), the same with --fast (folds the set's
//   items), a folded digest's text, and the too-small throw code.
#include <fstream>
#include <iostream>
#include <stdint.h>

#include "sdbf_class.h"
#include "sdbf_set.h"

int main(int argc, char** argv) {
    if (argc < 4) return 2;
    sdbf* a = new sdbf(argv[1], 0);
    sdbf* b = new sdbf(argv[2], 16 * 1024);
    std::cout << a;
    std::cout << b;
    std::cout << "a vs b " << a->compare(b, 0) << "\n";
    sdbf* a2 = new sdbf(a->to_string());
    sdbf* b2 = new sdbf(b->to_string());
    std::cout << "a2 vs b2 " << a2->compare(b2, 0) << "\n";
    std::ifstream is(argv[1], std::ios::binary);
    sdbf* a3 = new sdbf(argv[1], &is, 0, a->input_size(), NULL);
    std::cout << "istream equal " << (a3->to_string() == a->to_string()) << "\n";
    sdbf_set* set = new sdbf_set(argv[3]);
    std::cout << set->compare_all_quiet(1, 1, false);
    std::cout << set->compare_all_quiet(1, 1, true);
    std::cout << set->at(0);
    char small[100] = {0};
    try {
        sdbf tiny("tiny", small, 0, sizeof small, NULL);
    } catch (int e) {
        std::cout << "tiny throws " << e << "\n";
    }
    delete a;
    delete b;
    delete a2;
    delete b2;
    delete a3;
    for (uint32_t i = 0; i < set->size(); i++) delete set->at(i);
    delete set;
    return 0;
}
