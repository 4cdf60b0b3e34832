// Build-metadata strings that aphros normally generates from git at build
// time (src/gitrev -> util/gitgen.cpp).  The oracle build has no git
// metadata for the reference tree, so the values are fixed placeholders.
extern const char* kGitRev;
extern const char* kGitMsg;
extern const char* kGitDiff;
const char* kGitRev = "reference-oracle";
const char* kGitMsg = "";
const char* kGitDiff = "";
