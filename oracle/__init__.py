"""CPU oracle for libmat's RPD path -- test infrastructure, never product."""
