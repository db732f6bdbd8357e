/* Empty stand-in: the oracle build passes every switch with -D. */
