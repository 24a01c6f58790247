"""TEST INFRASTRUCTURE: the FP64 oracle of the Geliosphere SDE path and the
recipe that compiles the reference's own CPU code for pinning it.  Not part
of the product; see gelio_oracle.cpp."""
