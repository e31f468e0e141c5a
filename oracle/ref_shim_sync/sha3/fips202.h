/* empty: the reference includes this path; the functions come from the staged fips202.h */
