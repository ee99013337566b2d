// ingest.h -- FASTA text to the GPU.
//
// The species' files are read in large pieces of whole lines, cut only where a header
// line starts, so that no sequence spans two pieces; each piece is parsed on the device
// (blamm_stream_load_fasta) into the context's resident stream, whose run table gives
// the chunk markers the occurrence output needs.  Same stream, runs and sequence
// positions as FastaStream (FastaBatch, src/sequence.cpp:142-293), without the bases
// passing through host memory.  BLAMM_FASTA_READER=host selects FastaStream instead.
#pragma once

#include <cstdint>
#include <fstream>
#include <string>
#include <vector>

#include "sequence.h"

namespace blamm {

// true unless the environment sets BLAMM_FASTA_READER=host
bool gpuFastaReader();

// bytes per piece (BLAMM_INGEST_PIECE_BYTES, default 256 MiB)
size_t ingestPieceBytes();

class FastaPieceReader {
public:
    FastaPieceReader(std::vector<std::string> files, size_t pieceBytes);

    // The next piece: at least pieceBytes of text (the last one may be shorter), ending
    // where a header line starts or at the end of the files; a file without a final
    // newline gets one.  Returns false after the last piece.
    bool next(std::string &piece);

private:
    bool readMore();

    std::vector<std::string> files_;
    size_t fileIdx_ = 0, pieceBytes_;
    std::ifstream ifs_;
    bool lastNewline_ = true;
    std::string buf_;
};

// The first whitespace-delimited token of each header line (what `iss >> name` reads
// from the line after '>'), for header offsets into a piece's text.
std::vector<std::string> headerNames(const std::string &raw, const std::vector<int64_t> &headerPos);

// A resident stream's run table (stream position, sequence index, position in the
// sequence) as the markers of the chunk [begin, begin + size) with `payload` positions
// of its own; seqBase is added to the sequence indices.
void residentChunk(const std::vector<int64_t> &runStart, const std::vector<int64_t> &runSeq,
                   const std::vector<int64_t> &runSeqPos, int64_t begin, int64_t size, int64_t payload,
                   int64_t seqBase, StreamChunk &chunk);

}  // namespace blamm
