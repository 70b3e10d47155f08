// Drives the C++ adapter the way the reference's drivers drive their handlers
// (src/fgss.cu:88-116, src/bitmap.cu:98-121, src/hybrid.cu:133-161) and prints
// the pair counts:  adapter_join <sets file> <threshold>
// Without a GPU it prints "no device" and exits 0.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "hyset_gb300.hpp"

namespace hg = hyset_gb300;

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const double threshold = std::atof(argv[2]);
    try {
        hg::context ctx(0);
        const hg::host_collection hc = hg::read_collection(argv[1]);
        hg::device_collection dc(ctx, hc);
        const auto blocks = hg::make_blocks(hc, 64);

        auto pairs = std::make_shared<hg::output::pairs_handler>();
        hg::fgssjoin::handler fgss(ctx, dc, 64, false, threshold);
        fgss.setOutputHandler(pairs);
        fgss.join(blocks, blocks);

        auto count = std::make_shared<hg::output::count_handler>();
        hg::bitmap::handler bitmap(ctx, dc, 64, 64, true, threshold);
        bitmap.setOutputHandler(count);
        bitmap.join(blocks, blocks);

        const auto fast = hg::self_join(ctx, dc, threshold);

        // every length-compatible (probe, smaller id) pair through the candidate
        // verifier: the length filter a CPU filter applies first (Jaccard
        // minsize, similarity.hpp:44-46)
        auto verified = std::make_shared<hg::output::pairs_handler>();
        hg::hybrid::device_handler dh(ctx, dc, dc, 256, 2, false, 1024, 1u << 20, threshold);
        dh.setOutputHandler(verified);
        for (uint32_t p = 1; p < dc.size(); ++p) {
            std::vector<uint32_t> cands;
            const uint32_t minsize = (uint32_t)std::ceil(threshold * (double)hc.sizes[p]);
            for (uint32_t c = 0; c < p; ++c)
                if (hc.sizes[c] >= minsize) cands.push_back(c);
            dh.addCandidates(p, cands);
        }
        dh.flush();
        std::printf("fgss %lu bitmap %lu fast %zu verifier %lu\n", pairs->getCount(), count->getCount(), fast.size(),
                    verified->getCount());
    } catch (const hg::error& e) {
        if (e.status == HYSET_E_NODEVICE) {
            std::printf("no device\n");
            return 0;
        }
        std::fprintf(stderr, "error %d: %s\n", (int)e.status, e.what());
        return 1;
    }
    return 0;
}
