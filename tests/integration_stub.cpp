// integration_stub.cpp -- the replacement body of the reference's
// PWMScan::scanThreadCUBLAS (src/pwmscan.cpp:297-437) a maintainer would add to scan with
// include/blamm_gpu.h: resident motif bank, one blamm_scan call per sequence block, the
// reference's MotifOccurrence output.  tests/test_host_cpu.py compiles it against the
// reference's unmodified headers (syntax and types only).
#include "pwmscan.h"
#include "blamm_gpu.h"
using namespace std;

void PWMScan::scanThreadCUBLAS(int devID, size_t speciesID, ProgressIndicator& progInd,
                               FastaBatch& seqBatch)
{
const size_t overlap = motifContainer.getMaxMotifLen() - 1;
const size_t payload = settings.matrix_S_w * settings.matrix_S_h;  // the reference's block size
const Matrix& P = motifContainer.getMatrix();

blamm_ctx* ctx = nullptr;
if (blamm_ctx_create(devID, &ctx) != BLAMM_OK) throw runtime_error("blamm_ctx_create failed");
vector<int32_t> len(P.nCols());
vector<float> thr(P.nCols());
for (size_t c = 0; c < P.nCols(); c++) {
        const Motif& m = motifContainer[motifContainer.getMotifIDAtCol(c)];
        len[c] = (int32_t)m.size();
        thr[c] = m.getThreshold();
}
if (blamm_set_motifs(ctx, P.getData(), (int)P.nRows(), (int)P.nCols(), len.data(), thr.data()) != BLAMM_OK)
        throw runtime_error(blamm_last_error(ctx));

SeqBlock block;
vector<int64_t> runs;
vector<blamm_hit> hits(1 << 20);
vector<MotifOccurrence> occurrences;
while (seqBatch.getNextOverlappingBlock(block, payload, overlap)) {
        runs.clear();  // the block's run starts: marker to marker
        for (size_t p = 0; p < block.size(); p += block.getRemainingSeqLen(p))
                runs.push_back((int64_t)p);
        const string bases = block.substr(0, block.size());
        int64_t nHits = 0;
        int rc = blamm_scan(ctx, bases.data(), (int64_t)bases.size(), runs.data(), (int64_t)runs.size(),
                            hits.data(), (int64_t)hits.size(), &nHits);
        if (rc == BLAMM_ERR_OVERFLOW) {  // nHits holds the total: grow and rescan
                hits.resize((size_t)nHits);
                rc = blamm_scan(ctx, bases.data(), (int64_t)bases.size(), runs.data(), (int64_t)runs.size(),
                                hits.data(), (int64_t)hits.size(), &nHits);
        }
        if (rc != BLAMM_OK) throw runtime_error(blamm_last_error(ctx));
        for (int64_t i = 0; i < nHits; i++) {
                const blamm_hit& o = hits[(size_t)i];
                if ((size_t)o.pos >= payload) continue;  // the overlap belongs to the next block
                const SeqPos sp = block.getSeqPos((size_t)o.pos);
                const size_t motifID = motifContainer.getMotifIDAtCol((size_t)o.col);
                const char strand = motifContainer[motifID].isRevCompl() ? '-' : '+';
                occurrences.push_back(MotifOccurrence(motifID, speciesID, sp.getSeqIndex(),
                                                      sp.getSeqPos(), strand, o.score));
        }
        // unchanged from here: the reference's async writer hand-off of `occurrences`, its
        // clear() and the progress message (src/pwmscan.cpp:409-417); after the loop, its wait
        // for the writers (:420-423)
        (void)progInd;
        occurrences.clear();
}
blamm_ctx_destroy(ctx);
}
