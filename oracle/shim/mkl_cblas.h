/* Empty stand-in: the reference includes MKL headers in every TU but only its
   PARDISO/dgesv call sites need MKL, and those are replaced in the oracle build. */
