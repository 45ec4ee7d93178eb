"""TEST INFRASTRUCTURE ONLY: the CPU oracle for the BGZF -> columns path."""
