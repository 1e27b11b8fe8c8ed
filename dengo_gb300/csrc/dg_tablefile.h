/*
 * Reader and writer of the .dgt table bundle (dengo_gb300/tablefile.py)
 * (magic "DGTBL001", uint32 count, then per dataset: uint32 name length,
 * name, uint64 element count, float64 values; little-endian).  It replaces
 * the HDF5 reads of the reference (rates_and_rate_tables.C.template:278-304).
 */
#ifndef DG_TABLEFILE_H
#define DG_TABLEFILE_H

#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <string>
#include <utility>
#include <vector>

namespace dg {

inline bool read_table_file(const char *path, std::map<std::string, std::vector<double>> &out,
                            std::string &err)
{
    FILE *f = fopen(path, "rb");
    if (!f) {
        err = std::string("cannot open ") + path;
        return false;
    }
    char magic[8];
    uint32_t count = 0;
    bool ok = fread(magic, 1, 8, f) == 8 && memcmp(magic, "DGTBL001", 8) == 0 &&
              fread(&count, 4, 1, f) == 1;
    for (uint32_t i = 0; ok && i < count; i++) {
        uint32_t ln = 0;
        uint64_t n = 0;
        ok = fread(&ln, 4, 1, f) == 1 && ln < 4096;
        std::string name(ok ? ln : 0, '\0');
        ok = ok && fread(&name[0], 1, ln, f) == ln && fread(&n, 8, 1, f) == 1 &&
             n < (1ull << 32);
        std::vector<double> v(ok ? n : 0);
        ok = ok && fread(v.data(), 8, n, f) == n;
        if (ok) out[name] = std::move(v);
    }
    fclose(f);
    if (!ok) err = std::string("malformed table bundle ") + path;
    return ok;
}

/* Writes the named arrays as a .dgt bundle (the layout above). */
inline bool write_table_file(const char *path,
                             const std::vector<std::pair<std::string, std::vector<double>>> &sets,
                             std::string &err)
{
    FILE *f = fopen(path, "wb");
    if (!f) {
        err = std::string("cannot create ") + path;
        return false;
    }
    const uint32_t count = (uint32_t)sets.size();
    bool ok = fwrite("DGTBL001", 1, 8, f) == 8 && fwrite(&count, 4, 1, f) == 1;
    for (size_t i = 0; ok && i < sets.size(); i++) {
        const uint32_t ln = (uint32_t)sets[i].first.size();
        const uint64_t n = sets[i].second.size();
        ok = fwrite(&ln, 4, 1, f) == 1 && fwrite(sets[i].first.data(), 1, ln, f) == ln &&
             fwrite(&n, 8, 1, f) == 1 && fwrite(sets[i].second.data(), 8, n, f) == n;
    }
    ok = (fclose(f) == 0) && ok;
    if (!ok) err = std::string("cannot write ") + path;
    return ok;
}

}  // namespace dg
#endif
