// Dump files in the reference's format (src/dump.c:278-499): a sequence of
// files named from a template with one integer conversion (the file
// number), each holding a header, the system description and up to
// maxdumps FP32 records.  The header's record count is rewritten after
// every record, as dump() does, so a run that stops leaves a readable file.
//
// Layouts (host code, no device work):
//   native  the struct images an LP64 build of the reference writes with
//           fwrite: dump_mt (208 bytes: title[128], vsn[16], long istep,
//           long dump_interval, int dump_level, maxdumps, ndumps,
//           dump_size, unsigned long timestamp, dump_init,
//           restart_timestamp, sysinfo_size), dump_sysinfo_mt (float
//           deltat, int nmols, nmols_r, nspecies) with one 68-byte mol_mt
//           per species, then the records as floats, all little-endian
//           (src/structs.h:204-238);
//   XDR     the reference's XDR encoding (src/xdr.c:150-183): the same
//           fields big-endian, longs and unsigned longs as 4 bytes, strings
//           as fixed-length opaque data, "(XDR)" after the version.
// The version string is the one the reference's dump.c stamps ("2.27",
// the source revision after "$Revision: "), which its readers check
// (version 2.23 and later carry the per-species sysinfo).
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "moldy_gb300.h"

struct mdgpu_dumpfile {
   std::string tmpl, cur, err;
   std::string title;
   std::vector<mdgpu_dump_species> spec;
   mdgpu_dump_info info{};
   int dump_size = 0;
   int filenum = -1;            // file being written
   int ndumps = 0;              // records in it
   long total = 0;              // records in the sequence
   unsigned long file_stamp = 0;
   long file_istep = 0;
   std::FILE *f = nullptr;
};

namespace {

constexpr int L_NAME = 128, L_VSN = 16, L_SPEC = 32;
constexpr int MOL_BYTES = 4 * 6 + 4 * 3 + L_SPEC;   // mol_mt, 68

struct Buf {
   std::vector<unsigned char> b;
   bool xdr;
   void raw(const void *p, size_t n)
   {
      const unsigned char *c = static_cast<const unsigned char *>(p);
      b.insert(b.end(), c, c + n);
   }
   void u32(uint32_t v)
   {
      unsigned char c[4];
      for (int i = 0; i < 4; i++) c[i] = (unsigned char)(v >> (xdr ? 24 - 8 * i : 8 * i));
      raw(c, 4);
   }
   void u64(uint64_t v)   // native only
   {
      unsigned char c[8];
      for (int i = 0; i < 8; i++) c[i] = (unsigned char)(v >> (8 * i));
      raw(c, 8);
   }
   void i32(int v) { u32((uint32_t)v); }
   void f32(float v)
   {
      uint32_t u;
      std::memcpy(&u, &v, 4);
      u32(u);
   }
   // long / unsigned long: 8 bytes native (LP64), 4 bytes XDR (xdr_long)
   void lng(uint64_t v)
   {
      if (xdr) u32((uint32_t)v);
      else u64(v);
   }
};

// Accepts a template with at most one integer conversion (flags, width and
// precision allowed) and "%%" escapes; appends "%d" when it has none.
bool check_template(std::string &t, std::string &err)
{
   int nconv = 0;
   for (size_t i = 0; i < t.size(); i++) {
      if (t[i] != '%') continue;
      if (i + 1 < t.size() && t[i + 1] == '%') {
         i++;
         continue;
      }
      size_t j = i + 1;
      while (j < t.size() && std::strchr("-+ 0#", t[j])) j++;
      while (j < t.size() && t[j] >= '0' && t[j] <= '9') j++;
      if (j < t.size() && t[j] == '.') {
         j++;
         while (j < t.size() && t[j] >= '0' && t[j] <= '9') j++;
      }
      if (j >= t.size() || !std::strchr("diu", t[j])) {
         err = "dump file name: only an integer conversion (%d) is allowed";
         return false;
      }
      nconv++;
      i = j;
   }
   if (nconv > 1) {
      err = "dump file name: more than one conversion";
      return false;
   }
   if (nconv == 0) t += "%d";   // src/dump.c:318-319
   return true;
}

std::string file_name(const std::string &t, int n)
{
   char buf[4096];
   std::snprintf(buf, sizeof buf, t.c_str(), n);
   return buf;
}

void version(char *vsn, bool xdr)
{
   std::memset(vsn, 0, L_VSN);
   // strncpy of "2.27 $" then the terminator written over the space,
   // src/dump.c:404-405; XDR files append "(XDR)", src/dump.c:407-417
   std::memcpy(vsn, "2.27 $", 6);
   vsn[4] = '\0';
   if (xdr) std::memcpy(vsn + 4, "(XDR)", 5);
}

long sysinfo_bytes(int nspecies) { return 16 + (long)MOL_BYTES * nspecies; }

long header_bytes(bool xdr) { return xdr ? L_NAME + L_VSN + 6 * 4 + 4 * 4 : 208; }

std::vector<unsigned char> header(const mdgpu_dumpfile &d, bool with_sysinfo)
{
   const mdgpu_dump_info &I = d.info;
   Buf B{{}, I.xdr != 0};
   char title[L_NAME] = {0}, vsn[L_VSN];
   std::strncpy(title, d.title.c_str(), L_NAME - 1);
   version(vsn, B.xdr);
   B.raw(title, L_NAME);
   B.raw(vsn, L_VSN);
   B.lng((uint64_t)d.file_istep);
   B.lng((uint64_t)I.dump_interval);
   B.i32(I.dump_level);
   B.i32(I.maxdumps);
   B.i32(d.ndumps);
   B.i32(d.dump_size);
   B.lng(d.file_stamp);
   B.lng(I.dump_init);
   B.lng(d.ndumps ? I.restart_timestamp : 0);   // set when the first record is written
   B.lng((uint64_t)sysinfo_bytes(I.nspecies));
   if (with_sysinfo) {
      B.f32(I.deltat);
      B.i32(I.nmols);
      B.i32(I.nmols_r);
      B.i32(I.nspecies);
      for (const mdgpu_dump_species &m : d.spec) {
         for (int k = 0; k < 3; k++) B.f32(m.inertia[k]);
         B.f32(m.mass);
         B.f32(m.dipole);
         B.f32(m.charge);
         B.i32(m.nmols);
         B.i32(m.rdof);
         B.i32(m.framework);
         char nm[L_SPEC] = {0};
         std::strncpy(nm, m.name, L_SPEC - 1);
         B.raw(nm, L_SPEC);
      }
   }
   return B.b;
}

bool put(mdgpu_dumpfile *d, long pos, const std::vector<unsigned char> &b)
{
   if (std::fseek(d->f, pos, SEEK_SET) != 0 || std::fwrite(b.data(), 1, b.size(), d->f) != b.size()) {
      d->err = "write to dump file " + d->cur + " failed: " + std::strerror(errno);
      return false;
   }
   return true;
}

mdgpu_status start_file(mdgpu_dumpfile *d)
{
   if (d->f) {
      std::fclose(d->f);
      d->f = nullptr;
   }
   d->filenum++;
   d->cur = file_name(d->tmpl, d->filenum);
   if (std::FILE *e = std::fopen(d->cur.c_str(), "rb")) {
      std::fclose(e);
      d->err = "dump file " + d->cur + " exists already";
      return MDGPU_E_IO;
   }
   d->f = std::fopen(d->cur.c_str(), "w+b");
   if (!d->f) {
      d->err = "cannot open dump file " + d->cur + ": " + std::strerror(errno);
      return MDGPU_E_IO;
   }
   d->ndumps = 0;
   d->file_istep = d->info.istep + d->total * d->info.dump_interval;
   d->file_stamp = (unsigned long)std::time(nullptr);
   if (!put(d, 0, header(*d, true))) return MDGPU_E_IO;
   return MDGPU_OK;
}

}  // namespace

extern "C" mdgpu_status mdgpu_dump_open(mdgpu_dumpfile **out, const char *name_template, const mdgpu_dump_info *info)
{
   if (!out) return MDGPU_E_ARG;
   *out = nullptr;
   mdgpu_dumpfile *d = new (std::nothrow) mdgpu_dumpfile;
   if (!d) return MDGPU_E_NOMEM;
   *out = d;
   if (!name_template || !info || !info->species || info->nspecies < 1) {
      d->err = "NULL argument or no species";
      return MDGPU_E_ARG;
   }
   d->info = *info;
   d->title = info->title ? info->title : "";
   d->spec.assign(info->species, info->species + info->nspecies);
   d->info.species = d->spec.data();
   d->tmpl = name_template;
   if (!check_template(d->tmpl, d->err)) return MDGPU_E_ARG;
   d->dump_size = mdgpu_dump_size(info->dump_level, info->nmols, info->nmols_r);
   if (d->dump_size <= 0 || info->maxdumps < 1 || info->dump_interval < 1) {
      d->err = "dump level, maxdumps and dump interval must select records";
      return MDGPU_E_ARG;
   }
   if (d->info.dump_init == 0) d->info.dump_init = (unsigned long)std::time(nullptr);
   return MDGPU_OK;
}

extern "C" mdgpu_status mdgpu_dump_append(mdgpu_dumpfile *d, const float *record)
{
   if (!d || !record) return MDGPU_E_ARG;
   if (!d->f || d->ndumps >= d->info.maxdumps) {
      mdgpu_status s = start_file(d);
      if (s) return s;
   }
   const bool xdr = d->info.xdr != 0;
   Buf B{{}, xdr};
   B.b.reserve((size_t)d->dump_size * 4);
   for (int i = 0; i < d->dump_size; i++) B.f32(record[i]);
   const long pos = header_bytes(xdr) + sysinfo_bytes(d->info.nspecies) + (long)d->ndumps * d->dump_size * 4;
   if (!put(d, pos, B.b)) return MDGPU_E_IO;
   d->ndumps++;
   d->total++;
   if (!put(d, 0, header(*d, false))) return MDGPU_E_IO;
   if (std::fflush(d->f) != 0) {
      d->err = "flush of dump file " + d->cur + " failed: " + std::strerror(errno);
      return MDGPU_E_IO;
   }
   return MDGPU_OK;
}

extern "C" const char *mdgpu_dump_filename(const mdgpu_dumpfile *d) { return d ? d->cur.c_str() : ""; }

extern "C" const char *mdgpu_dump_errmsg(const mdgpu_dumpfile *d) { return d ? d->err.c_str() : "NULL handle"; }

extern "C" void mdgpu_dump_close(mdgpu_dumpfile *d)
{
   if (!d) return;
   if (d->f) std::fclose(d->f);
   delete d;
}
