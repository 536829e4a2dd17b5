/*
 * seqfile.h -- reader of the reference's pair files (">pattern" then
 * "<text", one sequence per line; utils/sequence_reader.cu:108-201) into one
 * buffer plus per-pair descriptors that point into it.
 */
#ifndef WFE_SEQFILE_H
#define WFE_SEQFILE_H

#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "wfe.h"

namespace wfe {

struct PairFile {
    char* data = nullptr;      /* the whole file (pinned when `pinned`) */
    size_t bytes = 0;
    bool pinned = false;
    wfe_pair* pairs = nullptr; /* descriptors into data (pinned when `pinned`) */
    size_t n = 0;              /* pairs read */
    uint32_t longest = 0;      /* longest sequence read */
    std::string error;         /* set when reading failed */

    PairFile() = default;
    PairFile(const PairFile&) = delete;
    PairFile& operator=(const PairFile&) = delete;
    ~PairFile();
};

/* Read up to max_pairs pairs from path with nthreads threads.  Lines are
 * terminated by '\n' (a '\r' before it is dropped); the first byte of a
 * pattern line must be '>' and of a text line '<' (utils/sequence_reader.cu:
 * 154-180).  When pin is set the buffers are page-locked so that the GPU can
 * read the sequences in place.  Returns false and sets pf.error on failure. */
bool read_pair_file(const std::string& path, size_t max_pairs, int nthreads, bool pin, PairFile& pf);

}  // namespace wfe

#endif
