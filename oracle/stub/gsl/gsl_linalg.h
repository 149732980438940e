/* Empty stand-in: part.c includes this header but the likelihood path uses none of it. */
