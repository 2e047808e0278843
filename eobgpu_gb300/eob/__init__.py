"""Drop-in mirror of the reference's `eob` package (see the top-level `eob`
alias): seobnrv4phm, new_Dormand_horiz, pyEOB, pydopr853, pytdinterp."""
