// Batch solution files as text on the GPU (cs_text.cu), called by the runtime.
#pragma once

struct CsTextArgs {
  const double *t, *y, *z, *p;  // device: t [T], y [T][ny], z at the nodes [T][nz], p [B][np]
  long long T;                  // node slots
  int B, ny, nz, np;
  const int *dN, *doff;         // device: nodes and first slot of every instance
  void* stream;
};

// Formats every value, sizes every file (offsets: B + 1 host entries) and,
// with out non-null and cap large enough, copies the files to out.
int cs_text_files(const CsTextArgs& a, char* out, long long cap, long long* offsets);
