// Bulk reader for the node and element blocks of an OOFEM text input deck
// (host code). The reference reads every record through its tokenizer and
// input-record objects (OOFEMTXTDataReader / OOFEMTXTInputRecord,
// src/core/oofemtxtdatareader.C, oofemtxtinputrecord.C) and instantiates one
// object per dof manager and element (Domain::instanciateYourself,
// src/core/domain.C:485-700); at 10^6 records that dominates the time to the
// first solve. Here one pass over the bytes of a block extracts what the device
// model needs -- the record number and one numeric array field (a node's
// `coords`, an element's `nodes`) -- into flat arrays, and flags records that
// carry further fields so the caller can read those few with its general
// record parser.
#include <ctype.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <string>
#include <thread>
#include <vector>

#include "internal.cuh"

namespace {

inline const char *skip_ws(const char *p, const char *end)
{
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
    return p;
}

inline const char *token_end(const char *p, const char *end)
{
    while (p < end && !(*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')) ++p;
    return p;
}

inline bool token_is(const char *a, const char *ae, const char *key)
{
    const size_t n = strlen(key);
    return (size_t)(ae - a) == n && strncasecmp(a, key, n) == 0;
}

}  // namespace

namespace {

struct Line {
    const char *b, *e;
};

// Parses one record line; returns "" on success, else the reason.
std::string parse_record(const Line &ln, const char *keyword, const char *field, int maxvals, int64_t *id_out,
                         double *vals, int32_t *nv_out, uint8_t *other_out)
{
    const char *q = skip_ws(ln.b, ln.e), *eol = ln.e;
    const char *te = token_end(q, eol);
    if (!token_is(q, te, keyword)) return std::string("expected a ") + keyword + " record";
    q = skip_ws(te, eol);
    // every number is parsed from inside its own line: strtod / strtol would
    // otherwise skip the newline and read the next record
    char *num_end = nullptr;
    errno = 0;
    const long long id = q < eol ? strtoll(q, &num_end, 10) : 0;
    if (q >= eol || num_end == q || errno) return "record number missing";
    q = skip_ws(num_end, eol);
    bool found = false, extra = false;
    while (q < eol) {
        te = token_end(q, eol);
        if (!found && token_is(q, te, field)) {
            q = skip_ws(te, eol);
            const long n = q < eol ? strtol(q, &num_end, 10) : -1;
            if (q >= eol || num_end == q || n < 0 || n > maxvals) return std::string("bad ") + field + " count";
            q = num_end;
            for (long k = 0; k < n; ++k) {
                q = skip_ws(q, eol);
                const double v = q < eol ? strtod(q, &num_end) : 0.0;
                if (q >= eol || num_end == q) return std::string("bad ") + field + " value";
                vals[k] = v;
                q = num_end;
            }
            *nv_out = (int32_t)n;
            found = true;
        } else {
            extra = true;   // another field: the caller parses this record in full
            q = te;
        }
        q = skip_ws(q, eol);
    }
    if (!found) return std::string("field ") + field + " missing";
    *id_out = id;
    *other_out = extra ? 1 : 0;
    return "";
}

}  // namespace

extern "C" {

int ogb_deck_parse_block(const char *path, int64_t offset, int64_t count, const char *keyword, const char *field,
                         int maxvals, int64_t *ids, double *vals, int32_t *nvals, uint8_t *other,
                         int64_t *next_offset, int64_t *lines)
{
    using namespace ogb;
    if (!path || !keyword || !field || count < 0 || maxvals <= 0 || offset < 0 || !next_offset)
        return fail(OGB_E_ARG, "null argument or negative size");
    if (count > 0 && (!ids || !vals || !nvals || !other)) return fail(OGB_E_ARG, "null output array");
    FILE *fh = fopen(path, "rb");
    if (!fh) return fail(OGB_E_ARG, std::string("cannot open ") + path);
    std::vector<char> buf;
    int rc = OGB_OK;
    if (fseek(fh, 0, SEEK_END) != 0) rc = fail(OGB_E_ARG, "cannot seek");
    const long size = rc == OGB_OK ? ftell(fh) : -1;
    if (rc == OGB_OK && (size < 0 || offset > size)) rc = fail(OGB_E_ARG, "offset beyond the end of the deck");
    if (rc == OGB_OK) {
        buf.resize((size_t)(size - offset) + 1);
        if (fseek(fh, (long)offset, SEEK_SET) != 0 ||
            fread(buf.data(), 1, (size_t)(size - offset), fh) != (size_t)(size - offset))
            rc = fail(OGB_E_ARG, "cannot read the deck");
        buf[buf.size() - 1] = '\n';
    }
    fclose(fh);
    if (rc != OGB_OK) return rc;
    // pass 1: the record lines of the block (blank and comment lines skipped)
    const char *p = buf.data(), *end = buf.data() + buf.size() - 1;
    std::vector<Line> recs;
    recs.reserve((size_t)count);
    int64_t nlines = 0;
    while ((int64_t)recs.size() < count) {
        if (p >= end) return fail(OGB_E_ARG, "deck ends inside a block of " + std::to_string(count) + " records");
        const char *eol = (const char *)memchr(p, '\n', (size_t)(end - p));
        if (!eol) eol = end;
        ++nlines;
        const char *q = skip_ws(p, eol);
        if (q != eol && *q != '#') recs.push_back({p, eol});
        p = eol + 1;
    }
    // pass 2: the records, in parallel over contiguous ranges
    const int64_t n = count;
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt < 1 ? 1 : (nt > 32 ? 32 : nt);
    if (n < 65536) nt = 1;
    std::vector<std::string> err(nt);
    std::vector<int64_t> err_rec(nt, -1);
    auto work = [&](unsigned t) {
        const int64_t r0 = n * t / nt, r1 = n * (t + 1) / nt;
        for (int64_t r = r0; r < r1; ++r) {
            std::string e = parse_record(recs[(size_t)r], keyword, field, maxvals, ids + r, vals + r * maxvals,
                                         nvals + r, other + r);
            if (!e.empty()) {
                err[t] = e;
                err_rec[t] = r;
                return;
            }
        }
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < nt; ++t) pool.emplace_back(work, t);
        for (auto &th : pool) th.join();
    }
    for (unsigned t = 0; t < nt; ++t)   // the first failing record of the block
        if (err_rec[t] >= 0)
            return fail(OGB_E_ARG, err[t] + " (record " + std::to_string(err_rec[t] + 1) + " of the block)");
    const int64_t consumed = (int64_t)(p - buf.data());
    *next_offset = offset + (consumed < (int64_t)size - offset ? consumed : (int64_t)size - offset);
    if (lines) *lines = nlines;
    return OGB_OK;
}

}  // extern "C"
