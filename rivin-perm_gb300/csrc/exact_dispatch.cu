// Dispatch over the compiled (order, group size, float rows) shapes of the
// exact kernel; key = N * 16 + G * 2 + FP.
#include "exact_glynn.cuh"

namespace pg {

bool exact_dispatch_0(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_1(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_2(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_3(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_4(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_5(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_6(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_7(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_8(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_9(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_10(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);
bool exact_dispatch_11(int, const ExactArgs *, int, cudaStream_t, cudaError_t *, int *);

static bool dispatch(int key, const ExactArgs *args, int blocks,
                     cudaStream_t stream, cudaError_t *err, int *occ) {
    if (exact_dispatch_0(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_1(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_2(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_3(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_4(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_5(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_6(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_7(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_8(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_9(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_10(key, args, blocks, stream, err, occ)) return true;
    if (exact_dispatch_11(key, args, blocks, stream, err, occ)) return true;
    return false;
}

bool exact_compiled(int N, int G, bool fp) {
    if (N < 2 || N > 48 || G < 1 || G > 7) return false;
    switch (N * 16 + G * 2 + (fp ? 1 : 0)) {
    case 34:
    case 36:
    case 50:
    case 52:
    case 54:
    case 66:
    case 68:
    case 70:
    case 72:
    case 71:
    case 73:
    case 82:
    case 84:
    case 86:
    case 88:
    case 87:
    case 89:
    case 98:
    case 100:
    case 102:
    case 104:
    case 103:
    case 105:
    case 114:
    case 116:
    case 118:
    case 120:
    case 119:
    case 121:
    case 130:
    case 132:
    case 134:
    case 136:
    case 135:
    case 137:
    case 146:
    case 148:
    case 150:
    case 152:
    case 151:
    case 153:
    case 162:
    case 164:
    case 166:
    case 168:
    case 167:
    case 169:
    case 178:
    case 180:
    case 182:
    case 184:
    case 183:
    case 185:
    case 194:
    case 196:
    case 198:
    case 200:
    case 199:
    case 201:
    case 210:
    case 212:
    case 214:
    case 216:
    case 215:
    case 217:
    case 226:
    case 228:
    case 230:
    case 232:
    case 231:
    case 233:
    case 242:
    case 244:
    case 246:
    case 248:
    case 247:
    case 249:
    case 258:
    case 260:
    case 262:
    case 264:
    case 263:
    case 265:
    case 276:
    case 278:
    case 280:
    case 279:
    case 281:
    case 292:
    case 294:
    case 296:
    case 295:
    case 297:
    case 308:
    case 310:
    case 312:
    case 311:
    case 313:
    case 324:
    case 326:
    case 328:
    case 327:
    case 329:
    case 340:
    case 342:
    case 344:
    case 343:
    case 345:
    case 356:
    case 358:
    case 360:
    case 359:
    case 361:
    case 372:
    case 374:
    case 376:
    case 375:
    case 377:
    case 388:
    case 390:
    case 392:
    case 394:
    case 396:
    case 391:
    case 393:
    case 395:
    case 397:
    case 404:
    case 406:
    case 408:
    case 410:
    case 412:
    case 407:
    case 409:
    case 411:
    case 413:
    case 420:
    case 422:
    case 424:
    case 426:
    case 428:
    case 423:
    case 425:
    case 427:
    case 429:
    case 436:
    case 438:
    case 440:
    case 442:
    case 444:
    case 439:
    case 441:
    case 443:
    case 445:
    case 452:
    case 454:
    case 456:
    case 458:
    case 460:
    case 455:
    case 457:
    case 459:
    case 461:
    case 468:
    case 470:
    case 472:
    case 474:
    case 476:
    case 471:
    case 473:
    case 475:
    case 477:
    case 484:
    case 486:
    case 488:
    case 490:
    case 492:
    case 487:
    case 489:
    case 491:
    case 493:
    case 500:
    case 502:
    case 504:
    case 506:
    case 508:
    case 503:
    case 505:
    case 507:
    case 509:
    case 516:
    case 518:
    case 520:
    case 522:
    case 524:
    case 519:
    case 521:
    case 523:
    case 525:
    case 534:
    case 536:
    case 538:
    case 540:
    case 535:
    case 537:
    case 539:
    case 541:
    case 550:
    case 552:
    case 554:
    case 556:
    case 551:
    case 553:
    case 555:
    case 557:
    case 566:
    case 568:
    case 570:
    case 572:
    case 567:
    case 569:
    case 571:
    case 573:
    case 582:
    case 584:
    case 586:
    case 588:
    case 583:
    case 585:
    case 587:
    case 589:
    case 598:
    case 600:
    case 602:
    case 604:
    case 599:
    case 601:
    case 603:
    case 605:
    case 614:
    case 616:
    case 618:
    case 620:
    case 615:
    case 617:
    case 619:
    case 621:
    case 630:
    case 632:
    case 634:
    case 636:
    case 631:
    case 633:
    case 635:
    case 637:
    case 646:
    case 648:
    case 650:
    case 652:
    case 647:
    case 649:
    case 651:
    case 653:
    case 662:
    case 664:
    case 666:
    case 668:
    case 663:
    case 665:
    case 667:
    case 669:
    case 678:
    case 680:
    case 682:
    case 684:
    case 679:
    case 681:
    case 683:
    case 685:
    case 694:
    case 696:
    case 698:
    case 700:
    case 695:
    case 697:
    case 699:
    case 701:
    case 710:
    case 712:
    case 714:
    case 716:
    case 711:
    case 713:
    case 715:
    case 717:
    case 726:
    case 728:
    case 730:
    case 732:
    case 727:
    case 729:
    case 731:
    case 733:
    case 742:
    case 744:
    case 746:
    case 748:
    case 743:
    case 745:
    case 747:
    case 749:
    case 758:
    case 760:
    case 762:
    case 764:
    case 759:
    case 761:
    case 763:
    case 765:
    case 774:
    case 776:
    case 778:
    case 780:
    case 775:
    case 777:
    case 779:
    case 781:
        return true;
    default:
        return false;
    }
}

cudaError_t launch_exact_any(int N, int G, bool fp, const ExactArgs &args, int blocks,
                             cudaStream_t stream) {
    cudaError_t err = cudaErrorInvalidValue;
    if (!dispatch(N * 16 + G * 2 + (fp ? 1 : 0), &args, blocks, stream, &err, nullptr))
        return cudaErrorInvalidValue;
    return err;
}

int occupancy_exact_any(int N, int G, bool fp) {
    cudaError_t err = cudaSuccess;
    int occ = 1;
    if (!dispatch(N * 16 + G * 2 + (fp ? 1 : 0), nullptr, 0, nullptr, &err, &occ)) return 1;
    return occ;
}

}  // namespace pg
