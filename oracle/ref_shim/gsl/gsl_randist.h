/* Empty stand-in: the propagator files use no GSL symbol. */
