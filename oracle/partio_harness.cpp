// PARTIO HARNESS -- test infrastructure, not product code.
//
// Writes and reads .bgeo files with partio's own code, compiled in place by
// oracle/build_ref.sh from the copy the reference vendors
// (extlib/include/partio: io/BGEO.cpp writeBGEO and readBGEO, io/ZIP.cpp,
// core/Particle*.cpp; nothing is copied). tests/test_bgeo_partio_cpu.py uses
// it to pin the library's .bgeo writer and reader to partio.
//
// sfpartio_write builds the particle set exactly as the reference's
// ExportBgeoFileCUDA does (seepage_flows/include/kiri_utils.h:364-448):
// attributes position (VECTOR 3), Cd (FLOAT 3), pscale (FLOAT 1) and label
// (INT 1), added in that order, then one particle per point; Partio::write
// on a ".bgeo" name calls writeBGEO uncompressed (io/ParticleIO.cpp:166-178),
// which is what this calls. sfpartio_read reads a file the way
// ReadBgeoFileForGPU does (kiri_utils.h:252-306): (x, y, z, pscale), the
// y / z swap on request, and pscale 0.01 when the file has none.
#include <Partio.h>
#include "io/readers.h"

#include <cstdint>
#include <iostream>
#include <sstream>

namespace Partio {
// core/ParticleCaching.cpp (linked for freeCached, which release() calls)
// refers to Partio::read of io/ParticleIO.cpp, which picks a reader by the
// file extension; this harness only reads .bgeo files, so read is readBGEO.
ParticlesDataMutable* read(const char* filename, const bool verbose, std::ostream& errorStream) {
    return readBGEO(filename, false, verbose ? &errorStream : nullptr);
}
}  // namespace Partio

extern "C" int sfpartio_write(const char* path, const float* pos, const float* col, const float* radius,
                              const int64_t* labels, int64_t n) {
    Partio::ParticlesDataMutable* p = Partio::create();
    Partio::ParticleAttribute position_attr = p->addAttribute("position", Partio::VECTOR, 3);
    Partio::ParticleAttribute color_attr = p->addAttribute("Cd", Partio::FLOAT, 3);
    Partio::ParticleAttribute pscale_attr = p->addAttribute("pscale", Partio::FLOAT, 1);
    Partio::ParticleAttribute label_attr = p->addAttribute("label", Partio::INT, 1);
    for (int64_t i = 0; i < n; ++i) {
        const int particle = p->addParticle();
        float* q = p->dataWrite<float>(position_attr, particle);
        float* c = p->dataWrite<float>(color_attr, particle);
        float* s = p->dataWrite<float>(pscale_attr, particle);
        int* l = p->dataWrite<int>(label_attr, particle);
        for (int k = 0; k < 3; ++k) {
            q[k] = pos[3 * i + k];
            c[k] = col[3 * i + k];
        }
        *s = radius[i];
        *l = int(labels[i]);
    }
    std::ostringstream err;
    const bool ok = Partio::writeBGEO(path, *p, false, &err);
    p->release();
    return ok ? 0 : 1;
}

// Returns the particle count (or -1 when partio cannot read the file);
// writes up to cap (x, y, z, pscale) records.
extern "C" int64_t sfpartio_read(const char* path, float* out4, int64_t cap, int flip_yz) {
    std::ostringstream err;
    Partio::ParticlesDataMutable* data = Partio::readBGEO(path, false, &err);
    if (!data) return -1;
    Partio::ParticleAttribute pos_attr, pscale_attr;
    if (!data->attributeInfo("position", pos_attr) ||
        (pos_attr.type != Partio::FLOAT && pos_attr.type != Partio::VECTOR) || pos_attr.count != 3) {
        data->release();
        return -1;
    }
    const bool has_pscale = data->attributeInfo("pscale", pscale_attr);
    const int64_t n = data->numParticles();
    for (int64_t i = 0; i < n && i < cap; ++i) {
        const float* q = data->data<float>(pos_attr, int(i));
        const float s = has_pscale ? *data->data<float>(pscale_attr, int(i)) : 0.01f;
        out4[4 * i] = q[0];
        out4[4 * i + 1] = flip_yz ? q[2] : q[1];
        out4[4 * i + 2] = flip_yz ? q[1] : q[2];
        out4[4 * i + 3] = s;
    }
    data->release();
    return n;
}
