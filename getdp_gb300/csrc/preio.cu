// Native text formatting of the two bulky blocks of a .pre file (host code
// only): the DOF records of $DofData (Dof_WriteFilePRE, DofData.cpp:363-462)
// and the rows of $ElementsXEdges (Geo_WriteFilePRE, GeoEntity.cpp:526-552).
// A record is "NumType Entity Harmonic 1 NumDof 1" for an unknown and
// "NumType Entity Harmonic 2 value 0" for a fixed DOF, the value printed as
// "%.16g" (LinAlg_PrintScalar); a row is "index width e_1 ... e_width".
// Integers go through std::to_chars, reals through std::to_chars with the
// general format at precision 16, which is specified to print as "%.16g" in
// the C locale.
#include <charconv>

#include "common.cuh"

namespace {

struct Out {
  char *p, *end;
  bool full = false;
  void put(char c)
  {
    if(p < end)
      *p++ = c;
    else
      full = true;
  }
  void put(long long v)
  {
    auto r = std::to_chars(p, end, v);
    if(r.ec != std::errc())
      full = true;
    else
      p = r.ptr;
  }
  void put_real(double v)
  {
    auto r = std::to_chars(p, end, v, std::chars_format::general, 16);
    if(r.ec != std::errc())
      full = true;
    else
      p = r.ptr;
  }
};

}  // namespace

extern "C" int gb300_format_dof_records(long long n, const long long *rec5, const double *val,
                                        char *out, long long cap, long long *len)
{
  if(n < 0 || (n > 0 && (!rec5 || !val)) || !out || !len || cap < 0) {
    gb::set_error("gb300_format_dof_records: bad arguments");
    return GB300_ERR_ARG;
  }
  Out o{out, out + cap};
  for(long long i = 0; i < n && !o.full; i++) {
    const long long *r = rec5 + 5 * i;
    o.put(r[0]);
    o.put(' ');
    o.put(r[1]);
    o.put(' ');
    o.put(r[2]);
    if(r[3] == 1) {
      o.put(' ');
      o.put('1');
      o.put(' ');
      o.put(r[4]);
      o.put(' ');
      o.put('1');
    }
    else {
      o.put(' ');
      o.put('2');
      o.put(' ');
      o.put_real(val[i]);
      o.put(' ');
      o.put('0');
    }
    o.put('\n');
  }
  if(o.full) {
    gb::set_error("gb300_format_dof_records: output buffer of %lld bytes too small", cap);
    return GB300_ERR_CAPACITY;
  }
  *len = o.p - out;
  return GB300_OK;
}

extern "C" int gb300_format_int_rows(long long nrows, int width, const long long *vals,
                                     long long first_index, char *out, long long cap,
                                     long long *len)
{
  if(nrows < 0 || width < 0 || (nrows > 0 && width > 0 && !vals) || !out || !len || cap < 0) {
    gb::set_error("gb300_format_int_rows: bad arguments");
    return GB300_ERR_ARG;
  }
  Out o{out, out + cap};
  for(long long i = 0; i < nrows && !o.full; i++) {
    o.put(first_index + i);
    o.put(' ');
    o.put((long long)width);
    if(width == 0) o.put(' ');  // "i 0 " as the row format writes it
    for(int k = 0; k < width; k++) {
      o.put(' ');
      o.put(vals[i * width + k]);
    }
    o.put('\n');
  }
  if(o.full) {
    gb::set_error("gb300_format_int_rows: output buffer of %lld bytes too small", cap);
    return GB300_ERR_CAPACITY;
  }
  *len = o.p - out;
  return GB300_OK;
}
