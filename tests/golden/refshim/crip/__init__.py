"""Stand-in for the ``crip`` package (only ``crip.io`` writers), for running the
reference's sources during fixture generation.  Test infrastructure only."""
