// Dispatch over the compiled (order, group size) pairs of the exact kernel,
// written by gen_exact_inst.py.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_1(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_2(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_3(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_4(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_5(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_6(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_7(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_8(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_9(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_10(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_11(int, int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);

static bool dispatch(int N, int G, const ExactArgs *args, int blocks,
                     cudaStream_t stream, cudaError_t *err, int *occ) {
    if (exact_dispatch_0(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_1(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_2(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_3(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_4(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_5(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_6(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_7(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_8(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_9(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_10(N, G, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_11(N, G, args, blocks, stream, err, occ)) return true;
    return false;
}

bool exact_compiled(int N, int G) {
    if (N < 2 || N > 48 || G < 1 || G > EXACT_MAX_G) return false;
    switch (N * 16 + G) {
    case 33:
    case 34:
    case 49:
    case 50:
    case 51:
    case 65:
    case 66:
    case 67:
    case 68:
    case 81:
    case 82:
    case 83:
    case 84:
    case 97:
    case 98:
    case 99:
    case 100:
    case 113:
    case 114:
    case 115:
    case 116:
    case 129:
    case 130:
    case 131:
    case 132:
    case 145:
    case 146:
    case 147:
    case 148:
    case 161:
    case 162:
    case 163:
    case 164:
    case 177:
    case 178:
    case 179:
    case 180:
    case 193:
    case 194:
    case 195:
    case 196:
    case 209:
    case 210:
    case 211:
    case 212:
    case 225:
    case 226:
    case 227:
    case 228:
    case 241:
    case 242:
    case 243:
    case 244:
    case 257:
    case 258:
    case 259:
    case 260:
    case 274:
    case 275:
    case 276:
    case 290:
    case 291:
    case 292:
    case 306:
    case 307:
    case 308:
    case 322:
    case 323:
    case 324:
    case 338:
    case 339:
    case 340:
    case 354:
    case 355:
    case 356:
    case 370:
    case 371:
    case 372:
    case 386:
    case 387:
    case 388:
    case 389:
    case 390:
    case 391:
    case 392:
    case 394:
    case 402:
    case 403:
    case 404:
    case 405:
    case 406:
    case 407:
    case 408:
    case 410:
    case 418:
    case 419:
    case 420:
    case 421:
    case 422:
    case 423:
    case 424:
    case 426:
    case 434:
    case 435:
    case 436:
    case 437:
    case 438:
    case 439:
    case 440:
    case 442:
    case 450:
    case 451:
    case 452:
    case 453:
    case 454:
    case 455:
    case 456:
    case 458:
    case 466:
    case 467:
    case 468:
    case 469:
    case 470:
    case 471:
    case 472:
    case 474:
    case 482:
    case 483:
    case 484:
    case 485:
    case 486:
    case 487:
    case 488:
    case 490:
    case 498:
    case 499:
    case 500:
    case 501:
    case 502:
    case 503:
    case 504:
    case 506:
    case 514:
    case 515:
    case 516:
    case 517:
    case 518:
    case 519:
    case 520:
    case 522:
    case 531:
    case 532:
    case 533:
    case 534:
    case 535:
    case 536:
    case 538:
    case 547:
    case 548:
    case 549:
    case 550:
    case 551:
    case 552:
    case 554:
    case 563:
    case 564:
    case 565:
    case 566:
    case 567:
    case 568:
    case 570:
    case 579:
    case 580:
    case 581:
    case 582:
    case 583:
    case 584:
    case 586:
    case 595:
    case 596:
    case 597:
    case 598:
    case 599:
    case 600:
    case 602:
    case 611:
    case 612:
    case 613:
    case 614:
    case 615:
    case 616:
    case 618:
    case 627:
    case 628:
    case 629:
    case 630:
    case 631:
    case 632:
    case 634:
    case 643:
    case 644:
    case 645:
    case 646:
    case 647:
    case 648:
    case 650:
    case 659:
    case 660:
    case 661:
    case 662:
    case 663:
    case 664:
    case 666:
    case 675:
    case 676:
    case 677:
    case 678:
    case 679:
    case 680:
    case 682:
    case 691:
    case 692:
    case 693:
    case 694:
    case 695:
    case 696:
    case 698:
    case 707:
    case 708:
    case 709:
    case 710:
    case 711:
    case 712:
    case 714:
    case 723:
    case 724:
    case 725:
    case 726:
    case 727:
    case 728:
    case 730:
    case 739:
    case 740:
    case 741:
    case 742:
    case 743:
    case 744:
    case 746:
    case 755:
    case 756:
    case 757:
    case 758:
    case 759:
    case 760:
    case 762:
    case 771:
    case 772:
    case 773:
    case 774:
    case 775:
    case 776:
    case 778:
        return true;
    default:
        return false;
    }
}

cudaError_t launch_exact_any(int N, int G, const ExactArgs &args, int blocks,
                             cudaStream_t stream) {
    cudaError_t err = cudaErrorInvalidValue;
    if (!dispatch(N, G, &args, blocks, stream, &err, nullptr)) return cudaErrorInvalidValue;
    return err;
}

int occupancy_exact_any(int N, int G) {
    cudaError_t err = cudaSuccess;
    int occ = 1;
    if (!dispatch(N, G, nullptr, 0, nullptr, &err, &occ)) return 1;
    return occ;
}

}  // namespace pg
