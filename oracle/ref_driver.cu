// ref_driver.cu — runs the REFERENCE's own host join code on the CPU.
//
// TEST INFRASTRUCTURE ONLY (pins the C restatement in oracle.c; produces the
// golden fixtures in tests/golden/).  Built by `make -C oracle ref` from the
// reference's headers where they lie; the output goes to oracle/_ref/ only.
//
//   ref_join <input.txt> <threshold> <allpairs|ppjoin> [whole|blocks] [block_size]
//
// Reads the input with hyset::collection::read_collection<jaccard>
// (include/hyset/collection.hpp:93-177), builds the inverted index on the CPU
// (the reference builds it with GPU kernels, include/hyset/index.hpp:251-282;
// this driver fills the same host_array_index layout: entries sorted by
// (token, setID), offsets[t] = end of list t), then calls
// hyset::algorithms::host::allpairs or ::ppjoin (host_algorithms.hpp:16-250)
// with a pairs_handler, as src/cpu_single.cu:116-136 does for "whole", and per
// length-filtered block pair as src/queue.cu:142-168 / :255-279 does for
// "blocks".  Prints "first second" per pair, then "# count N".
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include <hyset/collection.hpp>
#include <hyset/host_algorithms.hpp>
#include <hyset/index.hpp>
#include <hyset/output.hpp>
#include <hyset/similarity.hpp>
#include <hyset/structs.hpp>

template <typename Segment>
static hyset::index::host_array_index* cpu_index(Segment& seg, hyset::collection::host_collection& c) {
    unsigned int start = seg.first_entry_position();
    unsigned int end = seg.last_entry_position();
    unsigned int length = end - start;
    auto* ix = new hyset::index::host_array_index(c.universeSize, length > 0 ? length : 1);
    ix->index->length = length;
    std::vector<hyset::structs::entry> e(c.prefixes.begin() + start, c.prefixes.begin() + end);
    std::stable_sort(e.begin(), e.end(), hyset::structs::entry_comparator());
    for (unsigned int k = 0; k < c.universeSize; ++k) ix->offsets->at(k) = 0;
    for (auto& x : e) ix->offsets->at(x.token) += 1;
    unsigned int run = 0;
    for (unsigned int k = 0; k < c.universeSize; ++k) {
        run += ix->offsets->at(k);
        ix->offsets->at(k) = run;  // inclusive end of list k
    }
    for (unsigned int k = 0; k < length; ++k) ix->index->at(k) = e[k];
    return ix;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s input threshold allpairs|ppjoin [whole|blocks] [block]\n", argv[0]);
        return 2;
    }
    std::string input = argv[1];
    double threshold = std::atof(argv[2]);
    std::string algorithm = argv[3];
    std::string mode = argc > 4 ? argv[4] : "whole";
    unsigned int blockSize = argc > 5 ? (unsigned int)std::atoi(argv[5]) : 10000;

    hyset::collection::host_collection hostCollection;
    std::vector<hyset::structs::block> blocks =
        hyset::collection::read_collection<jaccard>(input, hostCollection, blockSize, threshold);

    std::shared_ptr<hyset::output::handler> out = std::make_shared<hyset::output::pairs_handler>();

    auto run = [&](auto* indexed, hyset::index::host_array_index* ix, auto* probe) {
        using Seg = typename std::remove_pointer<decltype(indexed)>::type;
        if (algorithm == "allpairs")
            hyset::algorithms::host::allpairs<Seg, hyset::index::host_array_index, jaccard>(
                indexed, hostCollection, ix, probe, hostCollection, out, threshold);
        else
            hyset::algorithms::host::ppjoin<Seg, hyset::index::host_array_index, jaccard>(
                indexed, hostCollection, ix, probe, hostCollection, out, threshold);
    };

    if (mode == "blocks") {
        for (auto& first : blocks) {
            hyset::index::host_array_index* ix = cpu_index(first, hostCollection);
            for (auto& second : blocks) {
                if (second.id < first.id) continue;
                unsigned int lastIndexedSize = hostCollection.sizes[first.endID];
                unsigned int firstProbeSize = hostCollection.sizes[second.startID];
                if (lastIndexedSize >= jaccard::minsize(firstProbeSize, threshold)) run(&first, ix, &second);
            }
            delete ix;
        }
    } else {
        hyset::structs::partition partition(0);
        for (auto& b : blocks) partition.blocks.push_back(&b);
        hyset::index::host_array_index* ix = cpu_index(partition, hostCollection);
        run(&partition, ix, &partition);
        delete ix;
    }

    auto* pairs = (hyset::output::pairs_handler*)out.get();
    for (auto& p : pairs->pairs) std::printf("%u %u\n", p.first, p.second);
    std::printf("# count %lu\n", (unsigned long)pairs->pairs.size());
    return 0;
}
